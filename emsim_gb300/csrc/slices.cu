// Slice-builder plan, atom binning and the generic (any size) slice build, with their
// C-ABI entry points (include/emsim_gb300.h).
//
// Replaces emsim::cuda::OneSliceBuilder / MultiSlicesBuilder
// (emsim/backend/cuda_ext/src/SliceBuilder.cu, SliceBuilder_kernel.cu) and the cupy
// band-limit + clip of emsim/backend/slice_builder_cuda.py:39-70, 88-99.
#include <cmath>
#include <vector>

#include "atoms_sort.h"
#include "binning.cuh"
#include "slice_plan.h"
#include "slices.h"
#include "wave_plan.h"

using namespace emsim_gb300;

namespace emsim_gb300 {

int check_slice_device(const emsim_gb300_slice_plan* p) {
    EMSIM_REQUIRE(p != nullptr, EMSIM_GB300_ERR_INVALID, "null slice plan");
    int dev = -1;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_REQUIRE(dev == p->device, EMSIM_GB300_ERR_DEVICE, "slice plan used on a device other than its own");
    return EMSIM_GB300_OK;
}

}  // namespace emsim_gb300

namespace {

int check_device(const emsim_gb300_slice_plan* p) { return check_slice_device(p); }

// numpy floor division (Python semantics) for the centred band-limit grid
inline int py_floordiv(int a, int b) {
    int q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}

// Full-spectrum real filter F(k) equivalent to the reference band-limit
// irfft2(rfft2(V) * fil[:, :n2//2+1]) (slice_builder_cuda.py:88-99): fil is the disc
// k1^2 + k2^2 <= (min(n1,n2)//2)^2 on numpy's centred grid arange(-n//2, -n//2 + n),
// ifftshifted.  C2R weights the stored half spectrum by w = 1 on self-conjugate
// columns and 2 elsewhere; for a real input this equals applying the symmetric
// F(k) = (G(k) + G(-k)) / 2 with G = w * fil on the half spectrum and 0 beyond it.
std::vector<float> bandlimit_full(int n1, int n2) {
    const int r = (n1 < n2 ? n1 : n2) / 2;
    auto centred = [](int i, int n) { return ((i + n / 2) % n) + py_floordiv(-n, 2); };
    const int h2 = n2 / 2;
    auto G = [&](int i, int j) -> double {
        if (j > h2) return 0.0;
        const int c1 = centred(i, n1), c2 = centred(j, n2);
        const double fil = ((long long)c1 * c1 + (long long)c2 * c2 <= (long long)r * r) ? 1.0 : 0.0;
        const bool selfconj = (j == 0) || (n2 % 2 == 0 && j == h2);
        return (selfconj ? 1.0 : 2.0) * fil;
    };
    std::vector<float> F((size_t)n1 * n2);
    for (int i = 0; i < n1; ++i)
        for (int j = 0; j < n2; ++j) {
            const int mi = (n1 - i) % n1, mj = (n2 - j) % n2;
            F[(size_t)i * n2 + j] = (float)(0.5 * (G(i, j) + G(mi, mj)));
        }
    return F;
}

int make_tw(int n, float2** out) {
    std::vector<float2> h(n);
    for (int m = 0; m < n; ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)n;
        h[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    EMSIM_CHECK_CUDA(cudaMalloc((void**)out, sizeof(float2) * n));
    EMSIM_CHECK_CUDA(cudaMemcpy(*out, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    return EMSIM_GB300_OK;
}

// ---------------------------------------------------------------------------------
// binning (CUDA rule of SliceBuilder_kernel.cu:9-123)
// ---------------------------------------------------------------------------------
constexpr int MAX_ELEMS = 128;

// One thread per atom.  Element of row r = number of cumulative counts <= r.  Counts
// accumulate as exact integers: float atomics of 1.0f while every bin stays below 2^24
// (guaranteed for n_atoms < 2^24), unsigned atomics plus a conversion pass otherwise, so
// the histogram never depends on execution order.
template <bool THREE_D, bool U32>
__global__ void bin_kernel(const float* __restrict__ coords, unsigned n_atoms, const uint32_t* __restrict__ counts,
                           int n_elems, BinAxis a0, BinAxis a1, BinAxis a2, float* out) {
    __shared__ unsigned long long cum[MAX_ELEMS];
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int e = 0; e < n_elems; ++e) {
            s += counts[e];
            cum[e] = s;
        }
    }
    __syncthreads();
    const long long plane = (long long)a1.n * a2.n;
    const long long vol = THREE_D ? plane * a0.n : plane;
    for (unsigned r = blockIdx.x * blockDim.x + threadIdx.x; r < n_atoms; r += gridDim.x * blockDim.x) {
        int lo = 0, hi = n_elems;  // first e with cum[e] > r
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (cum[mid] > r) hi = mid;
            else lo = mid + 1;
        }
        if (lo >= n_elems) continue;  // rows beyond sum(counts) belong to no element
        const float z = coords[3ull * r + 0], x = coords[3ull * r + 1], y = coords[3ull * r + 2];
        int i = 0, j = 0, k = 0;
        long long lin;
        if (THREE_D) {
            if (!bin_axis(z, a0, i) || !bin_axis(x, a1, j) || !bin_axis(y, a2, k)) continue;
            lin = (long long)lo * vol + (long long)i * plane + (long long)j * a2.n + k;
        } else {
            if (!bin_axis(x, a1, j) || !bin_axis(y, a2, k)) continue;
            lin = (long long)lo * vol + (long long)j * a2.n + k;
        }
        if (U32) atomicAdd(reinterpret_cast<unsigned*>(out) + lin, 1u);
        else atomicAdd(out + lin, 1.0f);
    }
}

__global__ void u32_to_f32_kernel(float* data, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        data[i] = (float)reinterpret_cast<unsigned*>(data)[i];
}

int bin_atoms(emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms, const uint32_t* counts, float* out,
              bool three_d, cudaStream_t st) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(out && (n_atoms == 0 || (coords && counts)), EMSIM_GB300_ERR_INVALID, "bin_atoms: bad arguments");
    EMSIM_REQUIRE(p->n_elems <= MAX_ELEMS, EMSIM_GB300_ERR_UNSUPPORTED, "bin_atoms: more than 128 elements");
    const long long plane = (long long)p->n1 * p->n2;
    const long long total = (three_d ? plane * p->n_slices : plane) * p->n_elems;
    EMSIM_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * total, st));
    if (n_atoms == 0) return EMSIM_GB300_OK;
    const BinAxis a0 = make_axis(p->n_slices, p->dz), a1 = make_axis(p->n1, p->d1), a2 = make_axis(p->n2, p->d2);
    int blocks = ceil_div(n_atoms, 256);
    if (blocks > 65535) blocks = 65535;
    const bool u32 = n_atoms >= (1u << 24);
    if (three_d) {
        if (u32) bin_kernel<true, true><<<blocks, 256, 0, st>>>(coords, n_atoms, counts, p->n_elems, a0, a1, a2, out);
        else bin_kernel<true, false><<<blocks, 256, 0, st>>>(coords, n_atoms, counts, p->n_elems, a0, a1, a2, out);
    } else {
        if (u32) bin_kernel<false, true><<<blocks, 256, 0, st>>>(coords, n_atoms, counts, p->n_elems, a0, a1, a2, out);
        else bin_kernel<false, false><<<blocks, 256, 0, st>>>(coords, n_atoms, counts, p->n_elems, a0, a1, a2, out);
    }
    EMSIM_CHECK_LAUNCH();
    if (u32) {
        int cb = ceil_div(total, 256);
        if (cb > 8192) cb = 8192;
        u32_to_f32_kernel<<<cb, 256, 0, st>>>(out, total);
        EMSIM_CHECK_LAUNCH();
    }
    return EMSIM_GB300_OK;
}

// ---------------------------------------------------------------------------------
// generic (any size) slice build: same algebra with direct DFTs
// ---------------------------------------------------------------------------------
__global__ void pack_pairs_kernel(SliceArgs a) {
    const long long npix = (long long)a.n1 * a.n2;
    const int img = blockIdx.y;
    const int e = img / a.n_pairs, pair = img - e * a.n_pairs;
    const int s0 = 2 * pair, s1 = 2 * pair + 1;
    const float* h0 = a.hist + ((long long)e * a.n_slices + s0) * npix;
    const float* h1 = s1 < a.n_slices ? a.hist + ((long long)e * a.n_slices + s1) * npix : nullptr;
    float2* z = a.work + (long long)img * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x)
        z[i] = make_float2(h0[i], h1 ? h1[i] : 0.f);
}

__global__ void element_sum_kernel(SliceArgs a) {
    const long long npix = (long long)a.n1 * a.n2;
    const int pair = blockIdx.y;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int e = 0; e < a.n_elems; ++e) {
            const float2 z = a.work[((long long)e * a.n_pairs + pair) * npix + i];
            const float w = a.filt[(long long)e * npix + i];
            acc.x = fmaf(w, z.x, acc.x);
            acc.y = fmaf(w, z.y, acc.y);
        }
        a.work[(long long)pair * npix + i] = acc;
    }
}

__global__ void unpack_clip_kernel(SliceArgs a) {
    const long long npix = (long long)a.n1 * a.n2;
    const int pair = blockIdx.y;
    const int s0 = 2 * pair, s1 = 2 * pair + 1;
    const float2* w = a.work + (long long)pair * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = w[i];
        a.out[(long long)s0 * npix + i] = v.x < 1e-13f ? 1e-13f : v.x;
        if (s1 < a.n_slices) a.out[(long long)s1 * npix + i] = v.y < 1e-13f ? 1e-13f : v.y;
    }
}

int generic_build(emsim_gb300_slice_plan* p, const SliceArgs& a, cudaStream_t st) {
    const long long npix = (long long)p->n1 * p->n2;
    int blocks = ceil_div(npix, 256);
    if (blocks > 2048) blocks = 2048;
    const int nz = a.n_elems * a.n_pairs;
    pack_pairs_kernel<<<dim3(blocks, nz), 256, 0, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    EMSIM_TRY(generic_dft_rows(a.work, a.work, p->n1, p->n2, false, p->tw2, nz, st));
    EMSIM_TRY(generic_dft_cols(a.work, p->n1, p->n2, false, p->tw1, nz, st));
    element_sum_kernel<<<dim3(blocks, a.n_pairs), 256, 0, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    EMSIM_TRY(generic_dft_cols(a.work, p->n1, p->n2, true, p->tw1, a.n_pairs, st));
    EMSIM_TRY(generic_dft_rows(a.work, a.work, p->n1, p->n2, true, p->tw2, a.n_pairs, st));
    unpack_clip_kernel<<<dim3(blocks, a.n_pairs), 256, 0, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// Workspace of build_slices for n_atoms atoms of n_img images, carved in this order
// (each piece 256-byte aligned).
struct AtomsWorkspace {
    size_t group_start, group_tmp, bucket, item, count, off, cursor, bucket_tmp, items, tile_counter, work, total;
    long long n_buckets;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// work_pairs: slice pairs per image held in the complex work buffer (-1: all of them)
AtomsWorkspace atoms_workspace(const emsim_gb300_slice_plan* p, unsigned n_atoms, int n_img, long long work_pairs = -1) {
    AtomsWorkspace w;
    const long long n_groups = (long long)n_img * p->n_elems;
    const long long pairs = (p->n_slices + 1) / 2;
    if (work_pairs < 0 || work_pairs > pairs) work_pairs = pairs;
    w.n_buckets = n_groups * pairs * p->n1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    w.group_start = take(sizeof(unsigned) * (n_groups + 1));
    w.group_tmp = take(sizeof(unsigned) * scan_tmp_words(n_groups));
    w.bucket = take(sizeof(unsigned) * (size_t)n_atoms);
    w.item = take(sizeof(unsigned) * (size_t)n_atoms);
    w.count = take(sizeof(unsigned) * (size_t)w.n_buckets);
    w.off = take(sizeof(unsigned) * ((size_t)w.n_buckets + 1));
    w.cursor = take(sizeof(unsigned) * (size_t)w.n_buckets);
    w.bucket_tmp = take(sizeof(unsigned) * scan_tmp_words(w.n_buckets));
    w.items = take(sizeof(unsigned) * (size_t)n_atoms);
    w.tile_counter = take(sizeof(unsigned));
    w.work = take(sizeof(float2) * (size_t)n_img * work_pairs * p->n1 * p->n2);
    w.total = o;
    return w;
}

// Counting sort of molecules given with atomic numbers (build_slices_z / _ragged and the
// chunked image) into the workspace's buckets; fills the bucket fields of a.
int bucket_atoms_z(emsim_gb300_slice_plan* p, const float* coords, const int32_t* z, unsigned n_atoms,
                   const uint32_t* atom_offsets, int n_mol, const float* shift, const int32_t* mol_slot,
                   const int32_t* elem_of_z, const int32_t* slot_slices, char* base, const AtomsWorkspace& w,
                   SliceArgs& a, cudaStream_t st) {
    auto U = [&](size_t off) { return reinterpret_cast<unsigned*>(base + off); };
    const long long pairs = (p->n_slices + 1) / 2;
    EMSIM_CHECK_CUDA(cudaMemsetAsync(U(w.count), 0, sizeof(unsigned) * (size_t)w.n_buckets, st));
    AtomBucketZArgs ba;
    ba.coords = coords;
    ba.z = z;
    ba.n_atoms = n_atoms;
    ba.atom_offsets = atom_offsets;
    ba.n_mol = n_mol;
    ba.shift = shift;
    ba.mol_slot = mol_slot;
    ba.elem_of_z = elem_of_z;
    ba.n_elems = p->n_elems;
    ba.n_pairs = (int)pairs;
    ba.n1 = p->n1;
    ba.ax0 = make_axis(p->n_slices, p->dz);
    ba.ax1 = make_axis(p->n1, p->d1);
    ba.ax2 = make_axis(p->n2, p->d2);
    ba.slot_slices = slot_slices;
    ba.bucket = U(w.bucket);
    ba.item = U(w.item);
    ba.bucket_count = U(w.count);
    EMSIM_TRY(atoms_bucket_z(ba, st));
    EMSIM_TRY(scan_u32(U(w.count), U(w.off), w.n_buckets, U(w.bucket_tmp), st));
    EMSIM_CHECK_CUDA(cudaMemcpyAsync(U(w.cursor), U(w.off), sizeof(unsigned) * (size_t)w.n_buckets,
                                     cudaMemcpyDeviceToDevice, st));
    EMSIM_TRY(atoms_scatter(U(w.bucket), U(w.item), n_atoms, U(w.cursor), U(w.items), st));
    a.work = reinterpret_cast<float2*>(base + w.work);
    a.filt = p->filt;
    a.tw = p->tw;
    a.n_elems = p->n_elems;
    a.n_slices = p->n_slices;
    a.n_pairs = (int)pairs;
    a.n1 = p->n1;
    a.n2 = p->n2;
    a.bucket_off = U(w.off);
    a.items = U(w.items);
    a.tile_counter = U(w.tile_counter);
    a.n_atoms = n_atoms;
    a.wq = p->wq;
    a.live_lo = p->col_cut + 1;
    a.live_hi = p->col_cut > 0 ? p->col_cut : 0;
    a.img_slices = slot_slices;
    return EMSIM_GB300_OK;
}

}  // namespace

extern "C" {

int emsim_gb300_slice_plan_create(const float* sf_half, int n_elems, int n_slices, int n1, int n2, double dz,
                                  double d1, double d2, int symmetric_bandlimit, emsim_gb300_slice_plan** plan) {
    EMSIM_REQUIRE(plan != nullptr, EMSIM_GB300_ERR_INVALID, "null plan output pointer");
    *plan = nullptr;
    EMSIM_REQUIRE(n_elems >= 1 && n_slices >= 1 && n1 >= 1 && n2 >= 1, EMSIM_GB300_ERR_INVALID,
                  "slice plan: sizes must be positive");
    EMSIM_REQUIRE(sf_half != nullptr, EMSIM_GB300_ERR_INVALID, "slice plan: null scattering factors");
    EMSIM_REQUIRE(d1 > 0 && d2 > 0 && dz > 0, EMSIM_GB300_ERR_INVALID, "slice plan: steps must be positive");
    EMSIM_REQUIRE(n1 <= 16384 && n2 <= 16384, EMSIM_GB300_ERR_UNSUPPORTED, "slice plan: side above 16384");
    auto* p = new emsim_gb300_slice_plan();
    p->n_elems = n_elems;
    p->n_slices = n_slices;
    p->n1 = n1;
    p->n2 = n2;
    p->dz = dz;
    p->d1 = d1;
    p->d2 = d2;
    p->fast = fast_len(n1) && fast_len(n2);
    auto fail = [&](int code) {
        cudaFree(p->tw1);
        cudaFree(p->tw2);
        cudaFree(p->filt);
        cudaFree(p->wq);
        delete p;
        return code;
    };
    if (cudaGetDevice(&p->device) != cudaSuccess) {
        set_error("cudaGetDevice failed");
        return fail(EMSIM_GB300_ERR_CUDA);
    }
    int st;
    if ((st = ensure_twiddles(p->device)) != EMSIM_GB300_OK) return fail(st);
    p->tw = twiddle_table();
    if (!p->fast) {
        if ((st = make_tw(n1, &p->tw1)) != EMSIM_GB300_OK) return fail(st);
        if ((st = make_tw(n2, &p->tw2)) != EMSIM_GB300_OK) return fail(st);
        // chirp tables of the Bluestein line transforms, built here rather than on first use
        if ((st = bluestein_prepare(n1)) != EMSIM_GB300_OK) return fail(st);
        if ((st = bluestein_prepare(n2)) != EMSIM_GB300_OK) return fail(st);
    }
    // T_e(k) = F(k) * SF_e(k) / N on the full spectrum; SF_e(k) = SF_e(-k) supplies the
    // columns beyond n2/2 from the stored half spectrum.
    const std::vector<float> F =
        symmetric_bandlimit ? bandlimit_full(n1, n2) : std::vector<float>((size_t)n1 * n2, 1.0f);
    const int h = n2 / 2 + 1;
    const double inv_n = 1.0 / ((double)n1 * (double)n2);
    std::vector<float> T((size_t)n_elems * n1 * n2);
    for (int e = 0; e < n_elems; ++e)
        for (int i = 0; i < n1; ++i)
            for (int j = 0; j < n2; ++j) {
                const float sf = j < h ? sf_half[((size_t)e * n1 + i) * h + j]
                                       : sf_half[((size_t)e * n1 + (n1 - i) % n1) * h + (n2 - j)];
                T[((size_t)e * n1 + i) * n2 + j] = (float)((double)F[(size_t)i * n2 + j] * (double)sf * inv_n);
            }
    // support of the filters along k2: T_e is even in k, so it is |k2| <= col_cut
    for (int j = 0; j < n2; ++j) {
        bool any = false;
        for (int e = 0; e < n_elems && !any; ++e)
            for (int i = 0; i < n1 && !any; ++i) any = T[((size_t)e * n1 + i) * n2 + j] != 0.0f;
        const int k2 = fftfreq_int(j, n2);
        const int ak = k2 < 0 ? -k2 : k2;
        if (any && ak > p->col_cut) p->col_cut = ak;
    }
    if (cudaMalloc((void**)&p->filt, sizeof(float) * T.size()) != cudaSuccess ||
        cudaMemcpy(p->filt, T.data(), sizeof(float) * T.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("slice plan: filter upload failed");
        return fail(EMSIM_GB300_ERR_CUDA);
    }
    if (p->fast) {
        // W^m (even slice of a pair) then i W^m (odd slice), 2^22-scaled fixed point
        std::vector<int2> wq(2 * (size_t)n2);
        for (int m = 0; m < n2; ++m) {
            const double ang = -2.0 * M_PI * (double)m / (double)n2;
            const int c = (int)std::llrint(std::cos(ang) * WQ_SCALE), s = (int)std::llrint(std::sin(ang) * WQ_SCALE);
            wq[m] = make_int2(c, s);
            wq[n2 + m] = make_int2(-s, c);
        }
        if (cudaMalloc((void**)&p->wq, sizeof(int2) * 2 * n2) != cudaSuccess ||
            cudaMemcpy(p->wq, wq.data(), sizeof(int2) * 2 * n2, cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("slice plan: fixed-point twiddle upload failed");
            return fail(EMSIM_GB300_ERR_CUDA);
        }
    }
    *plan = p;
    return EMSIM_GB300_OK;
}

int emsim_gb300_slice_plan_destroy(emsim_gb300_slice_plan* p) {
    if (!p) return EMSIM_GB300_OK;
    cudaFree(p->tw1);
    cudaFree(p->tw2);
    cudaFree(p->filt);
    cudaFree(p->wq);
    delete p;
    return EMSIM_GB300_OK;
}

int emsim_gb300_bin_atoms_one_slice(emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms,
                                    const uint32_t* counts, float* out, void* stream) {
    return bin_atoms(p, coords, n_atoms, counts, out, false, (cudaStream_t)stream);
}

int emsim_gb300_bin_atoms_multi_slices(emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms,
                                       const uint32_t* counts, float* out, void* stream) {
    return bin_atoms(p, coords, n_atoms, counts, out, true, (cudaStream_t)stream);
}

size_t emsim_gb300_make_slices_workspace_size(const emsim_gb300_slice_plan* p) {
    if (!p) return 0;
    const size_t pairs = (size_t)(p->n_slices + 1) / 2;
    return sizeof(float2) * (size_t)p->n_elems * pairs * p->n1 * p->n2;
}

size_t emsim_gb300_build_slices_workspace_size(const emsim_gb300_slice_plan* p, unsigned n_atoms, int n_batch) {
    if (!p || n_batch < 1) return 0;
    return atoms_workspace(p, n_atoms, n_batch).total;
}

int emsim_gb300_build_slices(emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms,
                             const uint32_t* elem_counts, int n_batch, float* out, void* workspace,
                             size_t workspace_bytes, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(p->fast, EMSIM_GB300_ERR_UNSUPPORTED,
                  "build_slices: slice side is not a power of two in [8, 4096]; use bin_atoms + make_slices");
    EMSIM_REQUIRE(n_batch >= 1 && out && elem_counts && workspace && (coords || n_atoms == 0),
                  EMSIM_GB300_ERR_INVALID, "build_slices: bad arguments");
    const AtomsWorkspace w = atoms_workspace(p, n_atoms, n_batch);
    EMSIM_REQUIRE(workspace_bytes >= w.total, EMSIM_GB300_ERR_INVALID, "build_slices: workspace too small");
    EMSIM_REQUIRE(((uintptr_t)workspace & 255) == 0, EMSIM_GB300_ERR_INVALID,
                  "build_slices: workspace not 256-byte aligned");
    EMSIM_REQUIRE(w.n_buckets < (long long)INVALID_BUCKET, EMSIM_GB300_ERR_UNSUPPORTED,
                  "build_slices: more than 2^32 - 1 (image, element, slice pair, row) buckets");
    const long long pairs = (p->n_slices + 1) / 2;
    EMSIM_REQUIRE((long long)n_batch * pairs <= 65535, EMSIM_GB300_ERR_UNSUPPORTED,
                  "build_slices: more than 65535 image x slice-pair planes per call");
    cudaStream_t st = (cudaStream_t)stream;
    char* base = (char*)workspace;
    auto U = [&](size_t off) { return reinterpret_cast<unsigned*>(base + off); };
    const int n_groups = n_batch * p->n_elems;
    EMSIM_TRY(scan_u32(elem_counts, U(w.group_start), n_groups, U(w.group_tmp), st));
    EMSIM_CHECK_CUDA(cudaMemsetAsync(U(w.count), 0, sizeof(unsigned) * (size_t)w.n_buckets, st));
    AtomBucketArgs ba;
    ba.coords = coords;
    ba.n_atoms = n_atoms;
    ba.group_start = U(w.group_start);
    ba.n_groups = n_groups;
    ba.n_pairs = (int)pairs;
    ba.n1 = p->n1;
    ba.ax0 = make_axis(p->n_slices, p->dz);
    ba.ax1 = make_axis(p->n1, p->d1);
    ba.ax2 = make_axis(p->n2, p->d2);
    ba.bucket = U(w.bucket);
    ba.item = U(w.item);
    ba.bucket_count = U(w.count);
    EMSIM_TRY(atoms_bucket(ba, st));
    EMSIM_TRY(scan_u32(U(w.count), U(w.off), w.n_buckets, U(w.bucket_tmp), st));
    EMSIM_CHECK_CUDA(cudaMemcpyAsync(U(w.cursor), U(w.off), sizeof(unsigned) * (size_t)w.n_buckets,
                                     cudaMemcpyDeviceToDevice, st));
    EMSIM_TRY(atoms_scatter(U(w.bucket), U(w.item), n_atoms, U(w.cursor), U(w.items), st));
    SliceArgs a;
    a.out = out;
    a.work = reinterpret_cast<float2*>(base + w.work);
    a.filt = p->filt;
    a.tw = p->tw;
    a.n_elems = p->n_elems;
    a.n_slices = p->n_slices;
    a.n_pairs = (int)pairs;
    a.n1 = p->n1;
    a.n2 = p->n2;
    a.n_img = n_batch;
    a.bucket_off = U(w.off);
    a.items = U(w.items);
    a.tile_counter = U(w.tile_counter);
    a.n_atoms = n_atoms;
    a.wq = p->wq;
    a.live_lo = p->col_cut + 1;
    a.live_hi = p->col_cut > 0 ? p->col_cut : 0;
    return slice_atoms_build(a, st);
}

int emsim_gb300_centralize(const float* coords, const int32_t* z, const uint32_t* atom_offsets, int n_mol,
                           float* shift_out, float* space_out, uint32_t* present_out, void* stream) {
    EMSIM_REQUIRE(n_mol >= 0 && atom_offsets && shift_out && space_out && (coords || n_mol == 0) &&
                      (present_out == nullptr || z != nullptr),
                  EMSIM_GB300_ERR_INVALID, "centralize: bad arguments");
    return centralize(coords, z, atom_offsets, n_mol, shift_out, space_out, present_out, (cudaStream_t)stream);
}

int emsim_gb300_build_slices_z(emsim_gb300_slice_plan* p, const float* coords, const int32_t* z, unsigned n_atoms,
                               const uint32_t* atom_offsets, int n_mol, const float* shift, const int32_t* mol_slot,
                               const int32_t* elem_of_z, int n_batch, float* out, void* workspace,
                               size_t workspace_bytes, void* stream) {
    return emsim_gb300_build_slices_ragged(p, coords, z, n_atoms, atom_offsets, n_mol, shift, mol_slot, elem_of_z,
                                           nullptr, n_batch, out, workspace, workspace_bytes, stream);
}

int emsim_gb300_build_slices_ragged(emsim_gb300_slice_plan* p, const float* coords, const int32_t* z,
                                    unsigned n_atoms, const uint32_t* atom_offsets, int n_mol, const float* shift,
                                    const int32_t* mol_slot, const int32_t* elem_of_z, const int32_t* slot_slices,
                                    int n_batch, float* out, void* workspace, size_t workspace_bytes, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(p->fast, EMSIM_GB300_ERR_UNSUPPORTED,
                  "build_slices_z: slice side is not a power of two in [8, 4096]; use bin_atoms + make_slices");
    EMSIM_REQUIRE(n_batch >= 1 && n_mol >= 1 && out && atom_offsets && shift && mol_slot && elem_of_z && workspace &&
                      ((coords && z) || n_atoms == 0),
                  EMSIM_GB300_ERR_INVALID, "build_slices_z: bad arguments");
    const AtomsWorkspace w = atoms_workspace(p, n_atoms, n_batch);
    EMSIM_REQUIRE(workspace_bytes >= w.total, EMSIM_GB300_ERR_INVALID, "build_slices_z: workspace too small");
    EMSIM_REQUIRE(((uintptr_t)workspace & 255) == 0, EMSIM_GB300_ERR_INVALID,
                  "build_slices_z: workspace not 256-byte aligned");
    EMSIM_REQUIRE(w.n_buckets < (long long)INVALID_BUCKET, EMSIM_GB300_ERR_UNSUPPORTED,
                  "build_slices_z: more than 2^32 - 1 (image, element, slice pair, row) buckets");
    const long long pairs = (p->n_slices + 1) / 2;
    EMSIM_REQUIRE((long long)n_batch * pairs <= 65535, EMSIM_GB300_ERR_UNSUPPORTED,
                  "build_slices_z: more than 65535 image x slice-pair planes per call");
    cudaStream_t st = (cudaStream_t)stream;
    SliceArgs a;
    EMSIM_TRY(bucket_atoms_z(p, coords, z, n_atoms, atom_offsets, n_mol, shift, mol_slot, elem_of_z, slot_slices,
                             (char*)workspace, w, a, st));
    a.out = out;
    a.n_img = n_batch;
    return slice_atoms_build(a, st);
}

// ---- image straight from atoms, slices built chunk by chunk ----------------------------
namespace {

struct ImageAtomsWorkspace {
    AtomsWorkspace atoms;  // buckets and the chunk's complex work buffer
    size_t slices, wave, total;
};

ImageAtomsWorkspace image_atoms_workspace(const emsim_gb300_slice_plan* p, unsigned n_atoms, int n_img,
                                          int chunk_pairs) {
    ImageAtomsWorkspace w;
    w.atoms = atoms_workspace(p, n_atoms, n_img, chunk_pairs);
    const size_t npix = (size_t)p->n1 * p->n2;
    size_t o = w.atoms.total;
    w.slices = o;
    o = align256(o + sizeof(float) * (size_t)n_img * 2 * chunk_pairs * npix);
    w.wave = o;
    o = align256(o + sizeof(float2) * (size_t)n_img * npix);
    w.total = o;
    return w;
}

int chunk_of(const emsim_gb300_slice_plan* p, int chunk_pairs) {
    const int pairs = (p->n_slices + 1) / 2;
    return chunk_pairs < 1 || chunk_pairs > pairs ? pairs : chunk_pairs;
}

}  // namespace

size_t emsim_gb300_image_from_atoms_workspace_size(const emsim_gb300_slice_plan* p, unsigned n_atoms, int n_batch,
                                                   int chunk_pairs) {
    if (!p || n_batch < 1) return 0;
    return image_atoms_workspace(p, n_atoms, n_batch, chunk_of(p, chunk_pairs)).total;
}

int emsim_gb300_image_from_atoms_z(emsim_gb300_slice_plan* p, emsim_gb300_wave_plan* wp, const float* coords,
                                   const int32_t* z, unsigned n_atoms, const uint32_t* atom_offsets, int n_mol,
                                   const float* shift, const int32_t* mol_slot, const int32_t* elem_of_z, int n_batch,
                                   double dose, double cs_mm, const double* defocus, int n_defocus, double aperture,
                                   float* image_out, int chunk_pairs, void* workspace, size_t workspace_bytes,
                                   void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_TRY(check_device(wp));
    EMSIM_REQUIRE(p->fast && wp->fast, EMSIM_GB300_ERR_UNSUPPORTED,
                  "image_from_atoms: sides must be powers of two in [8, 4096]");
    EMSIM_REQUIRE(wp->n1 == p->n1 && wp->n2 == p->n2, EMSIM_GB300_ERR_INVALID,
                  "image_from_atoms: wave plan and slice plan sizes differ");
    EMSIM_REQUIRE(n_batch >= 1 && n_mol >= 1 && image_out && atom_offsets && shift && mol_slot && elem_of_z &&
                      workspace && defocus && n_defocus >= 1 && ((coords && z) || n_atoms == 0),
                  EMSIM_GB300_ERR_INVALID, "image_from_atoms: bad arguments");
    const int chunk = chunk_of(p, chunk_pairs);
    const ImageAtomsWorkspace w = image_atoms_workspace(p, n_atoms, n_batch, chunk);
    EMSIM_REQUIRE(workspace_bytes >= w.total, EMSIM_GB300_ERR_INVALID, "image_from_atoms: workspace too small");
    EMSIM_REQUIRE(((uintptr_t)workspace & 255) == 0, EMSIM_GB300_ERR_INVALID,
                  "image_from_atoms: workspace not 256-byte aligned");
    EMSIM_REQUIRE(w.atoms.n_buckets < (long long)INVALID_BUCKET, EMSIM_GB300_ERR_UNSUPPORTED,
                  "image_from_atoms: more than 2^32 - 1 (image, element, slice pair, row) buckets");
    EMSIM_REQUIRE((long long)n_batch * chunk <= 65535, EMSIM_GB300_ERR_UNSUPPORTED,
                  "image_from_atoms: more than 65535 image x slice-pair planes per chunk");
    cudaStream_t st = (cudaStream_t)stream;
    char* base = (char*)workspace;
    SliceArgs a;
    EMSIM_TRY(bucket_atoms_z(p, coords, z, n_atoms, atom_offsets, n_mol, shift, mol_slot, elem_of_z, nullptr, base,
                             w.atoms, a, st));
    float* slices = reinterpret_cast<float*>(base + w.slices);
    float2* wave = reinterpret_cast<float2*>(base + w.wave);
    a.out = slices;
    a.n_img = n_batch;
    a.out_slices = 2 * chunk;
    const long long npix = (long long)p->n1 * p->n2;
    const float4* p1;
    const float2* p2;
    EMSIM_TRY(get_prop(wp, p->dz, st, &p1, &p2));
    RowArgs r = base_row(wp);
    r.out = wave;
    r.in = wave;
    r.slice_img_stride = 2LL * chunk * npix;
    r.const_val = make_float2((float)std::sqrt(dose * wp->d1 * wp->d2), 0.f);
    ColArgs c = base_col(wp, wave);
    c.p1 = p1;
    c.p2 = p2;
    for (int pair0 = 0; pair0 < a.n_pairs; pair0 += chunk) {
        a.pair0 = pair0;
        a.chunk_pairs = a.n_pairs - pair0 < chunk ? a.n_pairs - pair0 : chunk;
        EMSIM_TRY(slice_atoms_build(a, st));
        for (int s = 2 * pair0; s < p->n_slices && s < 2 * (pair0 + a.chunk_pairs); ++s) {
            r.slice = slices + (long long)(s - 2 * pair0) * npix;
            const int ops = s == 0 ? (ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT) : (ROW_IFFT | ROW_TRANSMIT | ROW_FFT);
            EMSIM_TRY(launch_row(p->n2, ops, r, n_batch, st));
            EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, c, n_batch, st));
        }
    }
    // FFT2(psi_exit) = n2 * FFT_cols(X): the lens acts on X directly with 1/n1
    for (int i0 = 0; i0 < n_batch; i0 += LENS_MAX) {
        const int cnt = n_batch - i0 < LENS_MAX ? n_batch - i0 : LENS_MAX;
        ColArgs cl = base_col(wp, wave + i0 * npix);
        set_lens(wp, cl, cs_mm, aperture, 1.0f / (float)p->n1);
        cl.n_c2 = n_defocus == 1 ? 1 : cnt;
        for (int j = 0; j < cl.n_c2; ++j) cl.c2v[j] = M_PI * wp->wave_length * defocus[(i0 + j) % n_defocus];
        EMSIM_TRY(launch_col(p->n1, COL_LENS, cl, cnt, st));
    }
    RowArgs ri = base_row(wp);
    ri.in = wave;
    ri.out_int = image_out;
    return launch_row(p->n2, ROW_IFFT | ROW_OUT_INTENSITY, ri, n_batch, st);
}

int emsim_gb300_make_slices(emsim_gb300_slice_plan* p, const float* hist, float* out, void* workspace,
                            size_t workspace_bytes, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(hist && out && workspace, EMSIM_GB300_ERR_INVALID, "make_slices: null pointer");
    EMSIM_REQUIRE(workspace_bytes >= emsim_gb300_make_slices_workspace_size(p), EMSIM_GB300_ERR_INVALID,
                  "make_slices: workspace too small");
    EMSIM_REQUIRE(((uintptr_t)workspace & 255) == 0, EMSIM_GB300_ERR_INVALID, "make_slices: workspace not 256-byte aligned");
    SliceArgs a;
    a.hist = hist;
    a.out = out;
    a.work = (float2*)workspace;
    a.filt = p->filt;
    a.tw = p->tw;
    a.n_elems = p->n_elems;
    a.n_slices = p->n_slices;
    a.n_pairs = (p->n_slices + 1) / 2;
    a.n1 = p->n1;
    a.n2 = p->n2;
    EMSIM_REQUIRE((long long)a.n_elems * a.n_pairs <= 65535, EMSIM_GB300_ERR_UNSUPPORTED,
                  "make_slices: more than 65535 element x slice-pair planes");
    cudaStream_t st = (cudaStream_t)stream;
    if (p->fast) return slice_fast_build(a, st);
    return generic_build(p, a, st);
}

}  // extern "C"
