// Counting sort of atoms into (image, element, slice pair, row) buckets.
#pragma once

#include "binning.cuh"
#include "engine.h"

namespace emsim_gb300 {

constexpr unsigned INVALID_BUCKET = 0xffffffffu;

struct AtomBucketArgs {
    const float* coords = nullptr;       // (n_atoms, 3) float32, columns (z, x, y)
    unsigned n_atoms = 0;
    const unsigned* group_start = nullptr;  // (n_groups + 1) exclusive prefix of per-(image, element) counts
    int n_groups = 0;                    // n_img * n_elems
    int n_pairs = 0, n1 = 0;
    BinAxis ax0, ax1, ax2;               // slice, row, column axes (CUDA rule)
    unsigned* bucket = nullptr;          // (n_atoms) bucket id or INVALID_BUCKET
    unsigned* item = nullptr;            // (n_atoms) (slice parity << 31) | column
    unsigned* bucket_count = nullptr;    // (n_buckets) zeroed before the call
};

// Unsorted variant: element from a Z lookup, molecule from atom offsets, coordinates
// shifted per molecule (centralisation) before binning.
struct AtomBucketZArgs {
    const float* coords = nullptr;      // (n_atoms, 3)
    const int* z = nullptr;             // (n_atoms) atomic numbers
    unsigned n_atoms = 0;
    const unsigned* atom_offsets = nullptr;  // (n_mol + 1) molecule m = atoms [off[m], off[m+1])
    int n_mol = 0;
    const float* shift = nullptr;       // (n_mol, 3) added to the coordinates (float32)
    const int* mol_slot = nullptr;      // (n_mol) output image of molecule m, -1 to skip
    const int* elem_of_z = nullptr;     // (128) element index of Z, -1 when absent
    int n_elems = 0, n_pairs = 0, n1 = 0;
    BinAxis ax0, ax1, ax2;
    // per output image: its own slice count (<= ax0.n); the slice axis of a molecule is
    // then the binning rule's axis for that count; nullptr: ax0 for every molecule
    const int* slot_slices = nullptr;
    unsigned* bucket = nullptr;
    unsigned* item = nullptr;
    unsigned* bucket_count = nullptr;
};

int atoms_bucket_z(const AtomBucketZArgs& a, cudaStream_t st);

// per molecule: shift = -r_min - (r_max - r_min) / 2 and the extent of the shifted
// coordinates, both float32 as emsim/atoms.py:37-47, 142-159 evaluate them; with
// present != nullptr also the 128-bit mask (4 words) of atomic numbers z present
int centralize(const float* coords, const int* z, const unsigned* atom_offsets, int n_mol, float* shift, float* space,
               unsigned* present, cudaStream_t st);

// exclusive scan of n unsigned values into out[0..n]; out[n] = total; tmp holds
// scan_tmp_words(n) words
size_t scan_tmp_words(long long n);
int scan_u32(const unsigned* in, unsigned* out, long long n, unsigned* tmp, cudaStream_t st);

int atoms_bucket(const AtomBucketArgs& a, cudaStream_t st);
int atoms_scatter(const unsigned* bucket, const unsigned* item, unsigned n_atoms, unsigned* cursor,
                  unsigned* items_out, cudaStream_t st);

}  // namespace emsim_gb300
