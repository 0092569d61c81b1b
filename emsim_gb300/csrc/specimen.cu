// Band-limit of specimen slices (emsim/tem.py:102-108, band_limit_specimen): each slice
// is low-passed with the disc (x - s1//2)^2 + (y - s2//2)^2 <= 4 r^2 / 9, r = min(s1, s2)//2,
// on numpy's centred grid (ifftshifted to the FFT grid, where the centred offsets are the
// fftfreq integers), and the real part is kept.  The reference transforms axes (0, 1) of
// the stack, which matches its own (n_slices, s1, s2) layout only for cubic stacks; here
// every slice of the (n_slices, s1, s2) stack is filtered on its lateral axes.
//
// Two slices travel as one complex image z = V_2p + i V_2p+1 (the mask is real and even,
// so the pair separates exactly): pack, row FFT, column pass with the mask as a separable
// table (the propagate mode with unit phase, per-row cutoff and 1/N), inverse row FFT,
// unpack.
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"

using namespace emsim_gb300;

namespace {

__global__ void pack_pairs_kernel(const float* s, float2* z, int n_slices, int n_pairs, long long npix) {
    const long long total = (long long)n_pairs * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / npix, pix = i - p * npix;
        const float a = s[(2 * p) * npix + pix];
        const float b = 2 * p + 1 < n_slices ? s[(2 * p + 1) * npix + pix] : 0.f;
        z[i] = make_float2(a, b);
    }
}

__global__ void unpack_pairs_kernel(const float2* z, float* out, int n_slices, int n_pairs, long long npix) {
    const long long total = (long long)n_pairs * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / npix, pix = i - p * npix;
        const float2 v = z[i];
        out[(2 * p) * npix + pix] = v.x;
        if (2 * p + 1 < n_slices) out[(2 * p + 1) * npix + pix] = v.y;
    }
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

}  // namespace

extern "C" {

size_t emsim_gb300_band_limit_workspace_size(int n_slices, int n1, int n2) {
    if (n_slices < 1 || n1 < 1 || n2 < 1) return 0;
    const size_t tables = ((size_t)n1 * sizeof(float4) + (size_t)n2 * sizeof(float2) + 255) / 256 * 256;
    return tables + (size_t)((n_slices + 1) / 2) * n1 * n2 * sizeof(float2);
}

int emsim_gb300_band_limit_slices(const float* slices, int n_slices, int n1, int n2, float* out, void* workspace,
                                  size_t workspace_bytes, void* stream) {
    EMSIM_REQUIRE(slices && out && workspace && n_slices >= 1, EMSIM_GB300_ERR_INVALID,
                  "band_limit_slices: bad arguments");
    EMSIM_REQUIRE(fast_len(n1) && fast_len(n2), EMSIM_GB300_ERR_UNSUPPORTED,
                  "band_limit_slices: sides must be powers of two between 8 and 4096");
    EMSIM_REQUIRE(workspace_bytes >= emsim_gb300_band_limit_workspace_size(n_slices, n1, n2),
                  EMSIM_GB300_ERR_INVALID, "band_limit_slices: workspace too small");
    EMSIM_REQUIRE(((uintptr_t)workspace & 255) == 0, EMSIM_GB300_ERR_INVALID,
                  "band_limit_slices: workspace not 256-byte aligned");
    int dev = 0;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_TRY(ensure_twiddles(dev));
    cudaStream_t st = (cudaStream_t)stream;
    const long long npix = (long long)n1 * n2;
    const int n_pairs = (n_slices + 1) / 2;
    // separable mask table: p1 = (1/N, 0, cutoff of row k1), p2 = (1, 0)
    const long long r = (n1 < n2 ? n1 : n2) / 2;
    std::vector<float4> p1(n1);
    std::vector<float2> p2(n2, make_float2(1.f, 0.f));
    const float inv_n = (float)(1.0 / (double)npix);
    for (int i = 0; i < n1; ++i) {
        const long long k1 = fftfreq_int(i, n1);
        long long c = -1;  // largest |k2| with 9 (k1^2 + k2^2) <= 4 r^2
        while (c + 1 <= n2 / 2 && 9 * (k1 * k1 + (c + 1) * (c + 1)) <= 4 * r * r) ++c;
        int ci = (int)c;
        float cf;
        std::memcpy(&cf, &ci, sizeof(cf));
        p1[i] = make_float4(inv_n, 0.f, cf, 0.f);
    }
    char* base = (char*)workspace;
    float4* d_p1 = reinterpret_cast<float4*>(base);
    float2* d_p2 = reinterpret_cast<float2*>(base + (size_t)n1 * sizeof(float4));
    float2* z = reinterpret_cast<float2*>(
        base + ((size_t)n1 * sizeof(float4) + (size_t)n2 * sizeof(float2) + 255) / 256 * 256);
    // pageable sources: the copies have taken the host data when the calls return
    EMSIM_CHECK_CUDA(cudaMemcpyAsync(d_p1, p1.data(), sizeof(float4) * n1, cudaMemcpyHostToDevice, st));
    EMSIM_CHECK_CUDA(cudaMemcpyAsync(d_p2, p2.data(), sizeof(float2) * n2, cudaMemcpyHostToDevice, st));
    pack_pairs_kernel<<<grid_for((long long)n_pairs * npix), 256, 0, st>>>(slices, z, n_slices, n_pairs, npix);
    EMSIM_CHECK_LAUNCH();
    RowArgs ra;
    ra.tw = twiddle_table();
    ra.err = error_word();
    ra.in = z;
    ra.out = z;
    ra.in_img_stride = ra.out_img_stride = npix;
    ra.n_rows = n1;
    EMSIM_TRY(launch_row(n2, ROW_FFT, ra, n_pairs, st));
    ColArgs ca;
    ca.tw = twiddle_table();
    ca.err = error_word();
    ca.data = z;
    ca.img_stride = npix;
    ca.n_rows = n1;
    ca.n_cols = n2;
    ca.p1 = d_p1;
    ca.p2 = d_p2;
    EMSIM_TRY(launch_col(n1, COL_PROPAGATE, ca, n_pairs, st));
    EMSIM_TRY(launch_row(n2, ROW_IFFT, ra, n_pairs, st));
    unpack_pairs_kernel<<<grid_for((long long)n_pairs * npix), 256, 0, st>>>(z, out, n_slices, n_pairs, npix);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

}  // extern "C"
