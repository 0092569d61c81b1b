// Counting sort of atoms into (image, element, slice pair, row) buckets, and the
// exclusive scan it needs.
//
// Every atom is binned with the reference's CUDA rule (binning.cuh) - the same integer
// (slice, row, column) the dense histogram uses - and becomes one 32-bit item
// (slice parity << 31 | row << 12 | column) in its bucket.  Bucket sizes come from integer atomics;
// the scatter places items with an atomic cursor, so the order inside a bucket is not
// fixed, but everything downstream only forms order-independent exact sums over a
// bucket (see slice_cols_atoms_kernel), which keeps the slices bit-deterministic.
#include "atoms_sort.h"

namespace emsim_gb300 {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

size_t scan_tmp_words(long long n) { return (size_t)((n + SCAN_CHUNK - 1) / SCAN_CHUNK) + 1; }

// block-wide exclusive scan of one value per thread; returns the exclusive prefix and
// writes the block total to *total
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* warp_sums, unsigned* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        unsigned s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    const unsigned warp_base = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[(blockDim.x >> 5) - 1];
    return warp_base + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_chunks_kernel(const unsigned* in, unsigned* out, long long n,
                                                                   unsigned* chunk_totals) {
    __shared__ unsigned warp_sums[32];
    const long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_ITEMS;
    unsigned v[SCAN_ITEMS];
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = base + i < n ? in[base + i] : 0u;
        s += v[i];
    }
    unsigned total;
    unsigned run = block_exclusive_scan(s, warp_sums, &total);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) chunk_totals[blockIdx.x] = total;
}

// one block: exclusive scan of the chunk totals in place, total of all to out[n]
__global__ void __launch_bounds__(SCAN_THREADS) scan_totals_kernel(unsigned* totals, int n_chunks, unsigned* out,
                                                                   long long n) {
    __shared__ unsigned warp_sums[32];
    unsigned carry = 0;
    for (int b0 = 0; b0 < n_chunks; b0 += SCAN_THREADS) {
        const int i = b0 + threadIdx.x;
        const unsigned v = i < n_chunks ? totals[i] : 0u;
        unsigned total;
        const unsigned ex = block_exclusive_scan(v, warp_sums, &total);
        if (i < n_chunks) totals[i] = carry + ex;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void add_chunk_offsets_kernel(unsigned* out, long long n, const unsigned* totals) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] += totals[i / SCAN_CHUNK];
}

int scan_u32(const unsigned* in, unsigned* out, long long n, unsigned* tmp, cudaStream_t st) {
    EMSIM_REQUIRE(n >= 0, EMSIM_GB300_ERR_INVALID, "scan: negative length");
    const int n_chunks = (int)((n + SCAN_CHUNK - 1) / SCAN_CHUNK);
    if (n_chunks == 0) {
        EMSIM_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned), st));
        return EMSIM_GB300_OK;
    }
    scan_chunks_kernel<<<n_chunks, SCAN_THREADS, 0, st>>>(in, out, n, tmp);
    EMSIM_CHECK_LAUNCH();
    scan_totals_kernel<<<1, SCAN_THREADS, 0, st>>>(tmp, n_chunks, out, n);
    EMSIM_CHECK_LAUNCH();
    if (n_chunks > 1) {
        int blocks = ceil_div(n, 256);
        if (blocks > 8192) blocks = 8192;
        add_chunk_offsets_kernel<<<blocks, 256, 0, st>>>(out, n, tmp);
        EMSIM_CHECK_LAUNCH();
    }
    return EMSIM_GB300_OK;
}

// per atom: group (image, element) from the prefix of per-group counts, bin, bucket id
__global__ void atoms_bucket_kernel(AtomBucketArgs a) {
    const long long plane = a.n1;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < (long long)a.n_atoms;
         r += (long long)gridDim.x * blockDim.x) {
        unsigned bk = INVALID_BUCKET, item = 0;
        if ((unsigned)r < a.group_start[a.n_groups]) {
            int lo = 0, hi = a.n_groups;  // first group g with start[g + 1] > r
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (a.group_start[mid + 1] > (unsigned)r) hi = mid;
                else lo = mid + 1;
            }
            const float z = a.coords[3 * r + 0], x = a.coords[3 * r + 1], y = a.coords[3 * r + 2];
            int s, i, j;
            if (bin_axis(z, a.ax0, s) && bin_axis(x, a.ax1, i) && bin_axis(y, a.ax2, j)) {
                bk = (unsigned)(((long long)lo * a.n_pairs + (s >> 1)) * plane + i);
                item = ((unsigned)(s & 1) << 31) | ((unsigned)i << 12) | (unsigned)j;
                atomicAdd(a.bucket_count + bk, 1u);
            }
        }
        a.bucket[r] = bk;
        a.item[r] = item;
    }
}

__global__ void atoms_scatter_kernel(const unsigned* bucket, const unsigned* item, unsigned n_atoms, unsigned* cursor,
                                     unsigned* items_out) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < (long long)n_atoms;
         r += (long long)gridDim.x * blockDim.x) {
        const unsigned bk = bucket[r];
        if (bk == INVALID_BUCKET) continue;
        items_out[atomicAdd(cursor + bk, 1u)] = item[r];
    }
}

__global__ void atoms_bucket_z_kernel(AtomBucketZArgs a) {
    const long long plane = a.n1;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < (long long)a.n_atoms;
         r += (long long)gridDim.x * blockDim.x) {
        unsigned bk = INVALID_BUCKET, item = 0;
        int lo = 0, hi = a.n_mol;  // molecule: first m with off[m + 1] > r
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (a.atom_offsets[mid + 1] > (unsigned)r) hi = mid;
            else lo = mid + 1;
        }
        const int zz = a.z[r];
        const int slot = lo < a.n_mol ? a.mol_slot[lo] : -1;
        const int e = (zz >= 0 && zz < 128) ? a.elem_of_z[zz] : -1;
        if (slot >= 0 && e >= 0) {
            const float* sh = a.shift + 3 * lo;
            const float z = __fadd_rn(a.coords[3 * r + 0], sh[0]);
            const float x = __fadd_rn(a.coords[3 * r + 1], sh[1]);
            const float y = __fadd_rn(a.coords[3 * r + 2], sh[2]);
            BinAxis az = a.ax0;
            if (a.slot_slices) {
                // the molecule's own slice axis, evaluated as the host's make_axis does
                int n = a.slot_slices[slot];
                n = n < 1 ? 1 : (n > a.ax0.n ? a.ax0.n : n);
                az.n = n;
                az.start = -az.d * floorf((float)(n + 1) / 2.0f);
                az.end = fmaf((float)n, az.d, az.start);
            }
            int s, i, j;
            if (bin_axis(z, az, s) && bin_axis(x, a.ax1, i) && bin_axis(y, a.ax2, j)) {
                bk = (unsigned)((((long long)slot * a.n_elems + e) * a.n_pairs + (s >> 1)) * plane + i);
                item = ((unsigned)(s & 1) << 31) | ((unsigned)i << 12) | (unsigned)j;
                atomicAdd(a.bucket_count + bk, 1u);
            }
        }
        a.bucket[r] = bk;
        a.item[r] = item;
    }
}

int atoms_bucket_z(const AtomBucketZArgs& a, cudaStream_t st) {
    if (a.n_atoms == 0) return EMSIM_GB300_OK;
    int blocks = ceil_div(a.n_atoms, 256);
    if (blocks > 16384) blocks = 16384;
    atoms_bucket_z_kernel<<<blocks, 256, 0, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// one block per molecule; min/max are exact, so the result does not depend on order.
// With z != nullptr also a 128-bit mask of the atomic numbers present (Z < 128).
__global__ void centralize_kernel(const float* coords, const int* z, const unsigned* off, float* shift, float* space,
                                  unsigned* present) {
    __shared__ float red[6][32];
    __shared__ unsigned mask[4];
    const int m = blockIdx.x;
    const unsigned a0 = off[m], a1 = off[m + 1];
    if (z) {
        if (threadIdx.x < 4) mask[threadIdx.x] = 0u;
        __syncthreads();
        for (unsigned r = a0 + threadIdx.x; r < a1; r += blockDim.x) {
            const int zz = z[r];
            if (zz >= 0 && zz < 128) atomicOr(&mask[zz >> 5], 1u << (zz & 31));
        }
        __syncthreads();
        if (threadIdx.x < 4) present[4 * m + threadIdx.x] = mask[threadIdx.x];
    }
    float sh[3];
    for (int pass = 0; pass < 2; ++pass) {
        float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (unsigned r = a0 + threadIdx.x; r < a1; r += blockDim.x) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v = coords[3ull * r + c];
                if (pass) v = __fadd_rn(v, sh[c]);
                mn[c] = fminf(mn[c], v);
                mx[c] = fmaxf(mx[c], v);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
                mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
            }
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                red[c][warp] = mn[c];
                red[3 + c][warp] = mx[c];
            }
        }
        __syncthreads();
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float lo = red[c][0], hi = red[3 + c][0];
            for (int w = 1; w < nw; ++w) {
                lo = fminf(lo, red[c][w]);
                hi = fmaxf(hi, red[3 + c][w]);
            }
            const float sp = __fsub_rn(hi, lo);  // r_max - r_min
            if (pass == 0) {
                sh[c] = __fsub_rn(-lo, sp * 0.5f);  // -r_min - space / 2.0
            } else if (threadIdx.x == 0) {
                shift[3 * m + c] = sh[c];
                space[3 * m + c] = sp;
            }
        }
        __syncthreads();
    }
}

int centralize(const float* coords, const int* z, const unsigned* atom_offsets, int n_mol, float* shift, float* space,
               unsigned* present, cudaStream_t st) {
    if (n_mol <= 0) return EMSIM_GB300_OK;
    centralize_kernel<<<n_mol, 256, 0, st>>>(coords, present ? z : nullptr, atom_offsets, shift, space, present);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

int atoms_bucket(const AtomBucketArgs& a, cudaStream_t st) {
    if (a.n_atoms == 0) return EMSIM_GB300_OK;
    int blocks = ceil_div(a.n_atoms, 256);
    if (blocks > 16384) blocks = 16384;
    atoms_bucket_kernel<<<blocks, 256, 0, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

int atoms_scatter(const unsigned* bucket, const unsigned* item, unsigned n_atoms, unsigned* cursor,
                  unsigned* items_out, cudaStream_t st) {
    if (n_atoms == 0) return EMSIM_GB300_OK;
    int blocks = ceil_div(n_atoms, 256);
    if (blocks > 16384) blocks = 16384;
    atoms_scatter_kernel<<<blocks, 256, 0, st>>>(bucket, item, n_atoms, cursor, items_out);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

}  // namespace emsim_gb300
