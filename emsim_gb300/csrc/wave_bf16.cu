// Split-BF16 tensor-core passes for 256-point transforms (the precision form of the
// multislice step).
//
// A 256-point DFT is two batched 16-point DFTs with a twiddle between them (four-step
// FFT, 256 = 16 x 16): for x[n1 + 16 n2],
//     Y[n1][k2] = sum_n2 x[n1 + 16 n2] W16^(n2 k2),   Y *= W256^(n1 k2),
//     X[k2 + 16 k1] = sum_n1 Y[n1][k2] W16^(n1 k1).
// Each 16-point stage over a tile of R = 8 vectors is one GEMM on the 5th-generation
// tensor cores: A = 128 rows (vector, index) x K = 32 (re/im of the 16 inputs), B = the
// 32 x 32 real form of the complex DFT matrix, D = 128 x 32 fp32 in tensor memory.  The
// operands are split into bf16 hi + lo parts (x = hi + lo, lo = bf16(x - hi)) and
// D = A_hi B_hi + A_hi B_lo + A_lo B_hi, accumulated in fp32 (the lo x lo term is below
// the bf16 product's rounding), which keeps about 16 significant bits per stage.
//
// Thread m of the CTA owns GEMM row m and tensor-memory lane m.  Stage A rows are
// m = row(r, n1) (vector r); stage B rows m = row(r, k2), so after stage B thread m holds
// X[k2 + 16 k1] for all k1 -- which, with 16 = 16, is exactly the stage-A row that the
// next transform (inverse after forward and back) needs: the passes chain the inverse
// and forward transforms with the pointwise multiply between them in registers.  The row
// pass uses row(r, i) = 16 r + i (a warp reads and writes 128 contiguous bytes of two
// rows), the column pass row(c, i) = 8 i + c (a warp covers eight adjacent columns).
//
// The inverse transform reuses the forward matrix: IDFT(x) = conj(DFT(conj(x))), and
// through the four steps the conjugations meet at the twiddle, so the inverse is "write
// conj(x), forward stage, forward twiddle, forward stage, read conj(D)" -- sign flips in
// registers only.
//
// Row pass (IFFT, transmit, FFT): vectors are 8 rows.  Column pass (FFT, propagate,
// IFFT): vectors are 8 consecutive columns.  Both gather and scatter straight to global
// memory (a warp's load touches 8 rows x 4 elements, or 4 rows x 8 columns), so a CTA's
// shared memory is only its operand tiles and tables and several CTAs per SM overlap
// their MMA latencies.  Both are persistent over tiles, allocate 32 tensor-memory
// columns per CTA once, and give up a bounded mbarrier wait by setting the device error
// word.
#include <cuda_bf16.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>

#include "engine.h"
#include "umma.cuh"
#include "wave_tma.cuh"

namespace emsim_gb300 {
namespace {

constexpr int N = 256, NS = 16, R = 8, THREADS = 128;
constexpr int KB = 2 * NS;                  // GEMM K and N (re/im of 16 points)
constexpr int K_BYTES = KB * 2;             // bf16 bytes per operand row
// K-major operand tiles without swizzle, padded so that neither the row writes nor the
// twiddle scatter meet bank conflicts: the four 8 x 16-byte core matrices of a row group
// sit LBO = 144 bytes apart (4 banks of skew), row groups SBO = 608 bytes apart (16
// banks of skew between groups two apart)
constexpr uint32_t LBO = 144, SBO = 608;
constexpr int A_BYTES = (128 / 8) * SBO;
constexpr int M_BYTES = (KB / 8) * SBO;
static_assert(3 * LBO + 128 <= SBO, "row groups overlap");

__host__ __device__ constexpr uint32_t kmajor(int r, int k) {
    return (uint32_t)((r >> 3) * SBO + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2);
}
constexpr uint32_t TMEM_COLS = 32;
constexpr int WAIT_WARPS = 1;

struct __align__(128) DftSmem {
    unsigned char a_hi[A_BYTES];
    unsigned char a_lo[A_BYTES];
    unsigned char fwd_hi[M_BYTES], fwd_lo[M_BYTES];
    float2 tw[NS * NS];  // tw[16 k2 + n1] = W256^(n1 k2): a warp's 16 n1 read 16 adjacent entries
    float4 p1[N];  // column pass: the propagator's row factors (ColArgs::p1)
    uint64_t bar;
    uint32_t tmem;
    int pad;
};

__device__ __forceinline__ void split2(float re, float im, __nv_bfloat162& hi, __nv_bfloat162& lo) {
    hi = __floats2bfloat162_rn(re, im);
    const float2 h = __bfloat1622float2(hi);
    lo = __floats2bfloat162_rn(re - h.x, im - h.y);
}

// DFT matrices and twiddles from the FP64-derived table exp(-2 pi i m / 4096)
__device__ void init_tables(DftSmem& s, const float2* __restrict__ tw4096) {
    for (int e = threadIdx.x; e < KB * KB; e += blockDim.x) {
        const int j = e / KB, i = e % KB;  // output column j = 2 k + c, input i = 2 n + p
        const int k = j >> 1, c = j & 1, n = i >> 1, p = i & 1;
        const float2 w = __ldg(tw4096 + ((n * k) & 15) * 256);  // W16^(n k)
        // out re: re_in * wr - im_in * wi ; out im: re_in * wi + im_in * wr
        const float vf = c == 0 ? (p == 0 ? w.x : -w.y) : (p == 0 ? w.y : w.x);
        const uint32_t off = kmajor(j, i);
        const __nv_bfloat16 fh = __float2bfloat16_rn(vf);
        *reinterpret_cast<__nv_bfloat16*>(s.fwd_hi + off) = fh;
        *reinterpret_cast<__nv_bfloat16*>(s.fwd_lo + off) = __float2bfloat16_rn(vf - __bfloat162float(fh));
    }
    for (int e = threadIdx.x; e < NS * NS; e += blockDim.x) {
        const int k2 = e >> 4, n1 = e & 15;
        s.tw[e] = __ldg(tw4096 + n1 * k2 * 16);
    }
}

// thread m writes its own GEMM row: 16 complex values (v[2n], v[2n + 1]), conjugated when
// CONJ, at K positions 2n, 2n + 1
template <bool CONJ>
__device__ __forceinline__ void write_row(DftSmem& s, int m, const float (&v)[KB]) {
#pragma unroll
    for (int g = 0; g < NS / 4; ++g) {  // 4 complex = 16 bytes = one core-matrix row
        __nv_bfloat162 h[4], l[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int n = 4 * g + q;
            split2(v[2 * n], CONJ ? -v[2 * n + 1] : v[2 * n + 1], h[q], l[q]);
        }
        const uint32_t off = kmajor(m, 8 * g);
        *reinterpret_cast<uint4*>(s.a_hi + off) = *reinterpret_cast<uint4*>(h);
        *reinterpret_cast<uint4*>(s.a_lo + off) = *reinterpret_cast<uint4*>(l);
    }
}

// GEMM row of (vector v, index i) in a tile of R = 8 vectors: VEC_MAJOR puts a vector's
// 16 indices in consecutive rows (m = 16 v + i: a warp covers two vectors, so its global
// accesses along a row are 128-byte contiguous), else m = 8 i + v (a warp covers eight
// vectors: eight consecutive columns)
template <bool VEC_MAJOR>
__device__ __forceinline__ int gemm_row(int v, int i) {
    return VEC_MAJOR ? 16 * v + i : 8 * i + v;
}
template <bool VEC_MAJOR>
__device__ __forceinline__ int row_vec(int m) {
    return VEC_MAJOR ? m >> 4 : m & 7;
}
template <bool VEC_MAJOR>
__device__ __forceinline__ int row_idx(int m) {
    return VEC_MAJOR ? m & 15 : m >> 3;
}

// stage-A output Y[n1][k2] of vector r (thread m = gemm_row(r, n1)) -> twiddle ->
// stage-B rows gemm_row(r, k2), K 2 n1
template <bool VEC_MAJOR>
__device__ __forceinline__ void twiddle_scatter(DftSmem& s, int m, const float (&d)[KB]) {
    const int n1 = row_idx<VEC_MAJOR>(m), r = row_vec<VEC_MAJOR>(m);
#pragma unroll
    for (int k2 = 0; k2 < NS; ++k2) {
        const float2 w = s.tw[NS * k2 + n1];
        const float re = d[2 * k2] * w.x - d[2 * k2 + 1] * w.y;
        const float im = d[2 * k2] * w.y + d[2 * k2 + 1] * w.x;
        __nv_bfloat162 h, l;
        split2(re, im, h, l);
        const uint32_t off = kmajor(gemm_row<VEC_MAJOR>(r, k2), 2 * n1);
        *reinterpret_cast<__nv_bfloat162*>(s.a_hi + off) = h;
        *reinterpret_cast<__nv_bfloat162*>(s.a_lo + off) = l;
    }
}

// one 16-point stage on the A tile: 6 MMAs (hi.hi, hi.lo, lo.hi over 2 K steps), then
// every thread reads its D row; false when the completion wait timed out
__device__ __forceinline__ bool stage(DftSmem& s, uint32_t& phase, float (&d)[KB], unsigned long long wait_ns) {
    tma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
        umma::fence_after_sync();
        const unsigned char* mh = s.fwd_hi;
        const unsigned char* ml = s.fwd_lo;
        constexpr uint32_t idesc = umma::idesc_bf16_f32(128, KB);
#pragma unroll
        for (int ks = 0; ks < KB / 16; ++ks) {
            const uint64_t ah = umma::smem_desc(s.a_hi + ks * 2 * LBO, LBO, SBO);
            const uint64_t al = umma::smem_desc(s.a_lo + ks * 2 * LBO, LBO, SBO);
            const uint64_t bh = umma::smem_desc(mh + ks * 2 * LBO, LBO, SBO);
            const uint64_t bl = umma::smem_desc(ml + ks * 2 * LBO, LBO, SBO);
            umma::mma_bf16(s.tmem, ah, bh, idesc, ks > 0 ? 1u : 0u);
            umma::mma_bf16(s.tmem, ah, bl, idesc, 1u);
            umma::mma_bf16(s.tmem, al, bh, idesc, 1u);
        }
        umma::commit(&s.bar);
    }
    // the first WAIT_WARPS warps wait for the completion (suspended, not spinning); the
    // others wait at the barrier
    const bool ok = threadIdx.x >= 32 * WAIT_WARPS || tma::mbar_wait_suspend(&s.bar, phase, wait_ns);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) return false;
    umma::fence_after_sync();
    const uint32_t base = umma::taddr(s.tmem, (threadIdx.x >> 5) * 32, 0);
#pragma unroll
    for (int c = 0; c < KB / 8; ++c) {
        float v[8];
        umma::ld_x8(base + 8 * c, v);
#pragma unroll
        for (int i = 0; i < 8; ++i) d[8 * c + i] = v[i];
    }
    umma::ld_wait();
    return true;
}

__device__ void setup(DftSmem& s, const float2* tw4096, const float4* p1 = nullptr) {
    if (threadIdx.x < 32) {
        umma::tmem_alloc(&s.tmem, TMEM_COLS);
        umma::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tma::mbar_init(&s.bar, 1);
        tma::fence_mbar_init();
    }
    init_tables(s, tw4096);
    if (p1)
        for (int m = threadIdx.x; m < N; m += blockDim.x) s.p1[m] = __ldg(p1 + m);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

// ok == false: a completion wait gave up; wait once more (bounded) for the MMAs in
// flight before the tensor memory is freed
__device__ void teardown(DftSmem& s, bool ok, uint32_t phase, unsigned long long wait_ns) {
    if (!ok) tma::mbar_drain(&s.bar, phase ^ 1u, wait_ns);
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) umma::tmem_dealloc(s.tmem, TMEM_COLS);
}

// ---- row pass: inverse row FFT, x exp(i sigma V), forward row FFT ----------------------
__global__ void __launch_bounds__(THREADS, 6) row_bf16_kernel(RowArgs a, int n_tiles) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    DftSmem& s = *reinterpret_cast<DftSmem*>(smem_raw);
    setup(s, a.tw);
    const int m = threadIdx.x;
    // row r of the tile; stage-A index n1 = lo4, stage-B index k2 = lo4
    const int r = row_vec<true>(m), lo4 = row_idx<true>(m);
    uint32_t phase = 0;
    bool ok = true;
    const int tiles_per_img = a.n_rows / R;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const long long img = tile / tiles_per_img;
        const int row = (tile - (int)img * tiles_per_img) * R + r;
        const float2* src = a.in + img * a.in_img_stride + (long long)row * N;
        const float* vsrc = a.slice + img * a.slice_img_stride + (long long)row * N;
        float d[KB], pot[NS];
#pragma unroll
        for (int n2 = 0; n2 < NS; ++n2) {
            const float2 v = src[lo4 + NS * n2];
            d[2 * n2] = v.x;
            d[2 * n2 + 1] = v.y;
        }
#pragma unroll
        for (int k1 = 0; k1 < NS; ++k1) pot[k1] = __ldg(vsrc + lo4 + NS * k1);  // used after the inverse
        write_row<true>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        twiddle_scatter<true>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        // thread (r, k2) holds conj(psi[k2 + 16 k1]): transmit, then it is the forward
        // transform's stage-A row (r, n1) with n1 = k2, n2 = k1
#pragma unroll
        for (int k1 = 0; k1 < NS; ++k1) {
            const float2 t = cmul(make_float2(d[2 * k1], -d[2 * k1 + 1]), transmit_factor(a.sigma_pi, pot[k1]));
            d[2 * k1] = t.x;
            d[2 * k1 + 1] = t.y;
        }
        write_row<false>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        twiddle_scatter<true>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        float2* dst = a.out + img * a.out_img_stride + (long long)row * N;
#pragma unroll
        for (int k1 = 0; k1 < NS; ++k1) dst[lo4 + NS * k1] = make_float2(d[2 * k1], d[2 * k1 + 1]);
    }
    if (!ok && m == 0) tma::record_error(a.err, tma::DEV_MBAR_TIMEOUT);
    teardown(s, ok, phase, a.wait_ns);
}

// ---- column pass: forward column FFT, x P(k) inside the band-limit / N, inverse --------
__global__ void __launch_bounds__(THREADS, 6) col_bf16_kernel(ColArgs a, int tiles_per_img, int lt_lo, int lt_hi,
                                                          int n_img) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    DftSmem& s = *reinterpret_cast<DftSmem*>(smem_raw);
    setup(s, a.tw, a.p1);
    const int m = threadIdx.x;
    // column c of the tile; stage-A index n1 = hi3, stage-B index k2 = hi3
    const int c = row_vec<false>(m), hi3 = row_idx<false>(m);
    uint32_t phase = 0;
    bool ok = true;
    const int live_per_img = lt_lo + lt_hi;
    const int n_tiles = live_per_img * n_img;
    const int ld = a.n_cols;  // (row, col) offsets below 2^31: 256 rows x n_cols
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int img = tile / live_per_img;
        const int j = tile - img * live_per_img;
        const int col = (j < lt_lo ? j : tiles_per_img - lt_hi + (j - lt_lo)) * R + c;
        float2* base = a.data + (long long)img * a.img_stride + col;
        float d[KB];
#pragma unroll
        for (int n2 = 0; n2 < NS; ++n2) {
            const float2 v = base[(hi3 + NS * n2) * ld];
            d[2 * n2] = v.x;
            d[2 * n2 + 1] = v.y;
        }
        write_row<false>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        twiddle_scatter<false>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        {
            // thread (c, k2) holds X[k] at k = k2 + 16 k1 of its column
            const int k2a = abs(fftfreq_int(col, a.n_cols));
            const float2 p2 = __ldg(a.p2 + col);
#pragma unroll
            for (int k1 = 0; k1 < NS; ++k1) {
                const float4 q = s.p1[hi3 + NS * k1];
                const float2 v = make_float2(d[2 * k1], d[2 * k1 + 1]);
                const float2 t = (k2a <= __float_as_int(q.z)) ? cmul(v, cmul(make_float2(q.x, q.y), p2))
                                                              : make_float2(0.f, 0.f);
                d[2 * k1] = t.x;
                d[2 * k1 + 1] = t.y;
            }
        }
        write_row<true>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
        twiddle_scatter<false>(s, m, d);
        if (!(ok = stage(s, phase, d, a.wait_ns))) break;
#pragma unroll
        for (int k1 = 0; k1 < NS; ++k1) base[(hi3 + NS * k1) * ld] = make_float2(d[2 * k1], -d[2 * k1 + 1]);
    }
    if (ok) {  // dead tiles: outside the band-limit in every row
        const int dead_per_img = tiles_per_img - live_per_img;
        for (int t = blockIdx.x; t < dead_per_img * n_img; t += gridDim.x) {
            const int img = t / dead_per_img;
            float2* base = a.data + (long long)img * a.img_stride + (lt_lo + t - img * dead_per_img) * R + c;
#pragma unroll
            for (int q = 0; q < N / 16; ++q) base[(hi3 + 16 * q) * ld] = make_float2(0.f, 0.f);
        }
    } else if (m == 0) {
        tma::record_error(a.err, tma::DEV_MBAR_TIMEOUT);
    }
    teardown(s, ok, phase, a.wait_ns);
}

constexpr size_t ROW_SMEM = sizeof(DftSmem);
constexpr size_t COL_SMEM = sizeof(DftSmem);

// Persistent grid of a tensor-memory kernel.  The occupancy API reports one resident CTA
// per SM for any kernel that allocates tensor memory, so residency is computed here from
// the kernel's registers and shared memory, the SM's limits and the 512 tensor-memory
// columns (TMEM_COLS per CTA).  A CTA beyond what fits waits for a slot, which costs
// time but not correctness: CTAs never wait on one another.
int tmem_grid(const void* func, size_t smem, int n_tiles) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find({dev, func});
        if (it != cache.end()) {
            per_sm = it->second;
        } else {
            cudaFuncAttributes fa{};
            int smem_sm = 0, regs_sm = 0, reserved = 0, thr_sm = 0, blk_sm = 0;
            cudaFuncGetAttributes(&fa, func);
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
            cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
            cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
            cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
            cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev);
            const int regs_cta = ((fa.numRegs + 7) / 8) * 8 * THREADS;
            per_sm = std::min(512 / (int)TMEM_COLS, thr_sm / THREADS);
            per_sm = std::min(per_sm, blk_sm);
            if (regs_cta > 0) per_sm = std::min(per_sm, regs_sm / regs_cta);
            per_sm = std::min(per_sm, (int)(smem_sm / (smem + fa.sharedSizeBytes + reserved)));
            if (per_sm < 1) per_sm = 1;
            cache[{dev, func}] = per_sm;
        }
    }
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    const long long g = std::min<long long>((long long)per_sm * std::max(n_sm, 1), n_tiles);
    return g < 1 ? 1 : (int)g;
}

}  // namespace

// 0: plain FP32 passes; 1: split-BF16 tensor-core passes where they exist (length 256)
static int g_precision = 0;

int precision_mode() { return g_precision; }

bool launch_row_bf16(int n2, int ops, const RowArgs& a, int n_img, cudaStream_t st, int* status) {
    if (g_precision != 1 || n2 != N || ops != (ROW_IFFT | ROW_TRANSMIT | ROW_FFT) || a.n_rows % R != 0) return false;
    const int n_tiles = (a.n_rows / R) * n_img;
    *status = ensure_smem_attr((const void*)row_bf16_kernel, ROW_SMEM);
    if (*status != EMSIM_GB300_OK) return true;
    const int grid = tmem_grid((const void*)row_bf16_kernel, ROW_SMEM, n_tiles);
    row_bf16_kernel<<<grid, THREADS, ROW_SMEM, st>>>(a, n_tiles);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("split-bf16 row pass launch: ") + cudaGetErrorString(e));
        *status = EMSIM_GB300_ERR_CUDA;
    } else {
        *status = EMSIM_GB300_OK;
    }
    return true;
}

bool launch_col_bf16(int n1, int mode, const ColArgs& a, int n_img, cudaStream_t st, int* status) {
    if (g_precision != 1 || n1 != N || mode != COL_PROPAGATE || a.n_cols % R != 0) return false;
    const int tiles_per_img = a.n_cols / R;
    const LiveTiles lt = live_tiles(a, R, tiles_per_img);
    *status = ensure_smem_attr((const void*)col_bf16_kernel, COL_SMEM);
    if (*status != EMSIM_GB300_OK) return true;
    const int grid = tmem_grid((const void*)col_bf16_kernel, COL_SMEM, tiles_per_img * n_img);
    col_bf16_kernel<<<grid, THREADS, COL_SMEM, st>>>(a, tiles_per_img, lt.lo, lt.hi, n_img);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("split-bf16 column pass launch: ") + cudaGetErrorString(e));
        *status = EMSIM_GB300_ERR_CUDA;
    } else {
        *status = EMSIM_GB300_OK;
    }
    return true;
}

}  // namespace emsim_gb300

extern "C" int emsim_gb300_set_precision(int mode) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(mode == 0 || mode == 1, EMSIM_GB300_ERR_INVALID,
                  "set_precision: 0 (plain FP32) or 1 (split-BF16 tensor-core passes)");
    g_precision = mode;
    return EMSIM_GB300_OK;
}

extern "C" int emsim_gb300_get_precision(void) { return emsim_gb300::precision_mode(); }
