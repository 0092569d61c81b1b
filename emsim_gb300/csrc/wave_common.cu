// Size dispatch of the fused passes, the twiddle table, the generic (any-size) path and
// the element-wise kernels of the wave propagator.
#include <atomic>
#include <mutex>
#include <set>
#include <utility>

#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>

#include <cudaTypedefs.h>

#include "wave_tma.cuh"

namespace emsim_gb300 {

// exp(-2 pi i m / TW_SIZE); one copy per device, written once by init_twiddle_kernel
static __device__ float2 g_twiddle[fft::TW_SIZE];
// error words: kernels record tma::DEV_MBAR_TIMEOUT in their device's word when a bounded
// wait gives up.  One int per device in mapped page-locked host memory, so that the host
// can read a word without synchronising the device (emsim_gb300_peek_device_error).
static int* g_err_host = nullptr;

// limit of the pipelined kernels' bounded waits (ns)
static std::atomic<unsigned long long> g_wait_limit_ns{tma::DEFAULT_WAIT_LIMIT_NS};
unsigned long long wait_limit_ns() { return g_wait_limit_ns.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------------
// error string (per host thread)
// ---------------------------------------------------------------------------------
static thread_local std::string t_last_error;
void set_error(const std::string& msg) { t_last_error = msg; }
const char* get_error() { return t_last_error.c_str(); }

// ---------------------------------------------------------------------------------
// one-time per-device state
// ---------------------------------------------------------------------------------
__global__ void init_twiddle_kernel() {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < fft::TW_SIZE) {
        double s, c;
        sincospi(-2.0 * (double)m / (double)fft::TW_SIZE, &s, &c);
        g_twiddle[m] = make_float2((float)c, (float)s);
    }
}

static std::mutex g_init_mu;
static std::set<int> g_twiddle_ready;
static const float2* g_twiddle_addr[64] = {};
static int* g_error_addr[64] = {};
static std::set<std::pair<int, const void*>> g_smem_ready;

// The table is written by a kernel on the legacy default stream and waited for, so it is
// visible to every stream of the device afterwards.  Called from plan creation.
int ensure_twiddles(int device) {
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_twiddle_ready.count(device)) return EMSIM_GB300_OK;
    EMSIM_REQUIRE(device >= 0 && device < 64, EMSIM_GB300_ERR_UNSUPPORTED, "device index above 63");
    init_twiddle_kernel<<<fft::TW_SIZE / 256, 256>>>();
    EMSIM_CHECK_LAUNCH();
    EMSIM_CHECK_CUDA(cudaDeviceSynchronize());
    void* addr = nullptr;
    EMSIM_CHECK_CUDA(cudaGetSymbolAddress(&addr, g_twiddle));
    g_twiddle_addr[device] = (const float2*)addr;
    if (!g_err_host) {
        EMSIM_CHECK_CUDA(cudaHostAlloc((void**)&g_err_host, 64 * sizeof(int),
                                       cudaHostAllocMapped | cudaHostAllocPortable));
        std::memset(g_err_host, 0, 64 * sizeof(int));
    }
    void* eaddr = nullptr;
    EMSIM_CHECK_CUDA(cudaHostGetDevicePointer(&eaddr, g_err_host + device, 0));
    g_error_addr[device] = (int*)eaddr;
    g_twiddle_ready.insert(device);
    return EMSIM_GB300_OK;
}

const float2* twiddle_table() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    return g_twiddle_addr[dev];
}

int* error_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    return g_error_addr[dev];
}

// ---------------------------------------------------------------------------------
// TMA support: persistent grid sizing and tensor maps
// ---------------------------------------------------------------------------------
bool tma_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("EMSIM_GB300_PASSES");
        return !(v && std::strcmp(v, "simple") == 0);
    }();
    return on;
}

bool pdl_enabled(cudaStream_t st) {
    static const int mode = [] {
        const char* v = std::getenv("EMSIM_GB300_PDL");
        return v ? std::atoi(v) : 1;
    }();
    if (mode <= 0) return false;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return false;
    return cap == cudaStreamCaptureStatusNone || mode >= 2;
}

static std::map<std::tuple<int, const void*, int, size_t>, int> g_occ;

int persistent_grid(const void* func, int threads, size_t smem, int n_tiles) {
    int dev = 0;
    cudaGetDevice(&dev);
    int per_sm = 0, n_sm = 0;
    {
        std::lock_guard<std::mutex> lk(g_init_mu);
        auto key = std::make_tuple(dev, func, threads, smem);
        auto it = g_occ.find(key);
        if (it != g_occ.end()) {
            per_sm = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem) != cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
            g_occ[key] = per_sm;
        }
    }
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    long long g = (long long)per_sm * (n_sm > 0 ? n_sm : 1);
    if (g > n_tiles) g = n_tiles;
    return g < 1 ? 1 : (int)g;
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

int make_col_tensor_map(CUtensorMap* map, const float2* data, long long n_rows_total, int n_cols, int box_cols,
                        int box_rows) {
    auto enc = tensor_map_encoder();
    EMSIM_REQUIRE(enc != nullptr, EMSIM_GB300_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)2 * n_cols, (cuuint64_t)n_rows_total};
    cuuint64_t strides[1] = {(cuuint64_t)n_cols * sizeof(float2)};
    cuuint32_t box[2] = {(cuuint32_t)(2 * box_cols), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(data), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    EMSIM_REQUIRE(r == CUDA_SUCCESS, EMSIM_GB300_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return EMSIM_GB300_OK;
}

int ensure_smem_attr(const void* func, size_t smem_bytes) {
    if (smem_bytes <= 48 * 1024) return EMSIM_GB300_OK;
    int dev = 0;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_init_mu);
    auto key = std::make_pair(dev, func);
    if (g_smem_ready.count(key)) return EMSIM_GB300_OK;
    EMSIM_CHECK_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    g_smem_ready.insert(key);
    return EMSIM_GB300_OK;
}

// ---------------------------------------------------------------------------------
// fast-path dispatch
// ---------------------------------------------------------------------------------
#define EMSIM_DECL(N)                                                                  \
    extern template int launch_row_n<N>(int, const RowArgs&, int, cudaStream_t);       \
    extern template int launch_col_n<N>(int, const ColArgs&, int, cudaStream_t);       \
    extern template int launch_row_tma_n<N>(int, const RowArgs&, int, cudaStream_t);   \
    extern template int launch_col_tma_n<N>(int, const ColArgs&, int, cudaStream_t);
EMSIM_FAST_SIZES(EMSIM_DECL)
#undef EMSIM_DECL


static int log2_fast(int n) {
    int k = 0;
    while ((1 << k) < n) ++k;
    return k;
}

// Built-in setting per length, as measured fastest on GB300 (µs per multislice step,
// TMA radix-8 against 16 values per thread): 256^2 x 16 images 18.9 / 15.2 (4 rows, 8
// columns per tile); 1024^2 x 8 96.8 / 84.6; 2048^2 x 1 63.5 / 54.7 (1 row per tile);
// 4096^2 x 1 277 / 207; at 512^2 the TMA radix-8 kernels win (19.6 / 20.6 x 4 images).
static PassTuning default_tuning(int n) {
    PassTuning t;
    switch (n) {
        case 256: t = {2, 4, 2, 8}; break;
        case 1024: t = {2, 0, 2, 0}; break;
        case 2048: t = {2, 1, 2, 0}; break;
        case 4096: t = {2, 0, 2, 0}; break;
        default: break;
    }
    return t;
}

// tuning table indexed by log2(n), n = 8 .. 4096
static PassTuning* tuning_table() {
    static PassTuning table[13];
    static bool init = [] {
        for (int k = 3; k <= 12; ++k) table[k] = default_tuning(1 << k);
        return true;
    }();
    (void)init;
    return table;
}
std::mutex g_tuning_mu;

PassTuning pass_tuning(int n) {
    if (!fast_len(n)) return PassTuning{};
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    return tuning_table()[log2_fast(n)];
}

int launch_row(int n2, int ops, const RowArgs& a, int n_img, cudaStream_t st) {
    int bf16_status;
    if (launch_row_bf16(n2, ops, a, n_img, st, &bf16_status)) return bf16_status;
    int r16_status;
    if (launch_row16(n2, ops, a, n_img, st, &r16_status)) return r16_status;
    const bool tma = tma_enabled() && n2 >= 16 && pass_tuning(n2).row_tma != 0 &&
                     ((ops & ROW_CONST_IN) || aligned16(a.in)) &&
                     (!(ops & ROW_TRANSMIT) || (aligned16(a.slice) && (a.slice_img_stride & 3) == 0));
    if (tma) {
        switch (n2) {
#define EMSIM_CASE(N) \
    case N: return launch_row_tma_n<N>(ops, a, n_img, st);
            EMSIM_FAST_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
        }
    }
    switch (n2) {
#define EMSIM_CASE(N) \
    case N: return launch_row_n<N>(ops, a, n_img, st);
        EMSIM_FAST_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
    }
    set_error("row pass: length not on the fast path");
    return EMSIM_GB300_ERR_UNSUPPORTED;
}

int launch_col(int n1, int mode, const ColArgs& a, int n_img, cudaStream_t st) {
    int bf16_status;
    if (launch_col_bf16(n1, mode, a, n_img, st, &bf16_status)) return bf16_status;
    int r16_status;
    if (launch_col16(n1, mode, a, n_img, st, &r16_status)) return r16_status;
    const bool tma = tma_enabled() && n1 >= 16 && pass_tuning(n1).col_tma != 0 && col_tma_B(n1, a.n_cols) >= 2 &&
                     aligned16(a.data);
    if (tma) {
        switch (n1) {
#define EMSIM_CASE(N) \
    case N: return launch_col_tma_n<N>(mode, a, n_img, st);
            EMSIM_FAST_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
        }
    }
    switch (n1) {
#define EMSIM_CASE(N) \
    case N: return launch_col_n<N>(mode, a, n_img, st);
        EMSIM_FAST_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
    }
    set_error("column pass: length not on the fast path");
    return EMSIM_GB300_ERR_UNSUPPORTED;
}

int row_tile(int n2) {
    int B = row_threads(n2) / (n2 / 8);
    return B;
}
int col_tile(int n1) { return col_B_for(n1, 1 << 30); }

// ---------------------------------------------------------------------------------
// generic path: direct DFT (O(n^2) per line) for lengths off the fast path
// ---------------------------------------------------------------------------------
// tw_n[m] = exp(-2 pi i m / n), m < n (FP64-derived).  One CTA per line.
__global__ void dft_rows_kernel(const float2* in, float2* out, int n_rows, int n, int inverse,
                                const float2* __restrict__ tw, long long img_stride) {
    extern __shared__ float2 line[];
    const long long img = blockIdx.y;
    const long long off = img * img_stride + (long long)blockIdx.x * n;
    for (int j = threadIdx.x; j < n; j += blockDim.x) line[j] = in[off + j];
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        long long idx = 0;
        for (int j = 0; j < n; ++j) {
            float2 w = __ldg(tw + idx);
            if (inverse) w.y = -w.y;
            acc = cadd(acc, cmul(line[j], w));
            idx += k;
            if (idx >= n) idx -= n;
        }
        // every thread has read the whole row into smem before any write (in-place safe)
        out[off + k] = acc;
    }
}

__global__ void dft_cols_kernel(float2* data, int n_rows, int n_cols, int inverse,
                                const float2* __restrict__ tw, long long img_stride) {
    extern __shared__ float2 line[];
    const long long img = blockIdx.y;
    float2* base = data + img * img_stride + blockIdx.x;
    const int n = n_rows;
    for (int j = threadIdx.x; j < n; j += blockDim.x) line[j] = base[(long long)j * n_cols];
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        long long idx = 0;
        for (int j = 0; j < n; ++j) {
            float2 w = __ldg(tw + idx);
            if (inverse) w.y = -w.y;
            acc = cadd(acc, cmul(line[j], w));
            idx += k;
            if (idx >= n) idx -= n;
        }
        // every thread has read the whole column into smem before any write
        base[(long long)k * n_cols] = acc;
    }
}

int generic_dft_rows(const float2* in, float2* out, int n_rows, int n, bool inverse, const float2* tw_n,
                     int n_img, cudaStream_t st) {
    int status;
    if (bluestein_rows(in, out, n_rows, n, inverse, n_img, st, &status)) return status;
    const size_t smem = (size_t)n * sizeof(float2);
    EMSIM_TRY(ensure_smem_attr((const void*)dft_rows_kernel, smem));
    dft_rows_kernel<<<dim3(n_rows, n_img), 256, smem, st>>>(in, out, n_rows, n, inverse ? 1 : 0, tw_n,
                                                            (long long)n_rows * n);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

int generic_dft_cols(float2* data, int n_rows, int n_cols, bool inverse, const float2* tw_n, int n_img,
                     cudaStream_t st) {
    int status;
    if (bluestein_cols(data, n_rows, n_cols, inverse, n_img, st, &status)) return status;
    const size_t smem = (size_t)n_rows * sizeof(float2);
    EMSIM_TRY(ensure_smem_attr((const void*)dft_cols_kernel, smem));
    dft_cols_kernel<<<dim3(n_cols, n_img), 256, smem, st>>>(data, n_rows, n_cols, inverse ? 1 : 0, tw_n,
                                                            (long long)n_rows * n_cols);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// ---------------------------------------------------------------------------------
// element-wise kernels
// ---------------------------------------------------------------------------------
__global__ void transmit_kernel(const float2* in, const float* __restrict__ slice, float2* out, long long n,
                                float sigma_pi, long long in_stride, long long slice_stride, long long out_stride) {
    const long long img = blockIdx.y;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[img * out_stride + i] = cmul(in[img * in_stride + i], transmit_factor(sigma_pi, slice[img * slice_stride + i]));
}

int ew_transmit(const float2* in, const float* slice, float2* out, long long n, float sigma_pi, int n_img,
                long long in_stride, long long slice_stride, long long out_stride, cudaStream_t st) {
    int blocks = ceil_div(n, 256);
    if (blocks > 4096) blocks = 4096;
    transmit_kernel<<<dim3(blocks, n_img), 256, 0, st>>>(in, slice, out, n, sigma_pi, in_stride, slice_stride,
                                                         out_stride);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

__global__ void fill_kernel(float2* out, long long n, float2 value) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = value;
}

int ew_fill(float2* out, long long n, float2 value, cudaStream_t st) {
    int blocks = ceil_div(n, 256);
    if (blocks > 8192) blocks = 8192;
    fill_kernel<<<blocks, 256, 0, st>>>(out, n, value);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

__global__ void intensity_kernel(const float2* __restrict__ in, float* __restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        out[i] = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
    }
}

int ew_intensity(const float2* in, float* out, long long n, cudaStream_t st) {
    int blocks = ceil_div(n, 256);
    if (blocks > 8192) blocks = 8192;
    intensity_kernel<<<blocks, 256, 0, st>>>(in, out, n);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

__global__ void axpy_kernel(float* __restrict__ y, const float* __restrict__ x, float a, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = fmaf(a, x[i], y[i]);
}

int ew_axpy(float* y, const float* x, float a, long long n, cudaStream_t st) {
    int blocks = ceil_div(n, 256);
    if (blocks > 8192) blocks = 8192;
    axpy_kernel<<<blocks, 256, 0, st>>>(y, x, a, n);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// full-spectrum multiply by P(k) * band-limit (p1 carries 1/N), for the generic path
__global__ void propagate_kernel(float2* data, ColArgs a) {
    const long long n = (long long)a.n_rows * a.n_cols;
    const long long img = blockIdx.y;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / a.n_cols), c = (int)(i - (long long)r * a.n_cols);
        const float4 q = a.p1[r];
        float2* p = data + img * a.img_stride + i;
        const bool keep = abs(fftfreq_int(c, a.n_cols)) <= __float_as_int(q.z);
        *p = keep ? cmul(*p, cmul(make_float2(q.x, q.y), a.p2[c])) : make_float2(0.f, 0.f);
    }
}

int ew_propagate(float2* data, const ColArgs& a, int n_img, cudaStream_t st) {
    int blocks = ceil_div((long long)a.n_rows * a.n_cols, 256);
    if (blocks > 4096) blocks = 4096;
    propagate_kernel<<<dim3(blocks, n_img), 256, 0, st>>>(data, a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

__global__ void lens_kernel(float2* data, ColArgs a) {
    const long long n = (long long)a.n_rows * a.n_cols;
    const long long img = blockIdx.y;
    const double c2 = a.c2v[a.n_c2 > 1 ? img : 0];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / a.n_cols), c = (int)(i - (long long)r * a.n_cols);
        const int k2 = fftfreq_int(c, a.n_cols);
        const double fy = (double)k2 * a.dfy64;
        float2* p = data + img * a.img_stride + i;
        *p = cmul(*p, lens_factor(fftfreq_int(r, a.n_rows), k2, fy * fy, c2, a));
    }
}

int ew_lens(float2* data, const ColArgs& a, int n_img, cudaStream_t st) {
    int blocks = ceil_div((long long)a.n_rows * a.n_cols, 256);
    if (blocks > 4096) blocks = 4096;
    lens_kernel<<<dim3(blocks, n_img), 256, 0, st>>>(data, a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// p1[k1] = {exp(-i phase_coef fx^2) * inv_n, band-limit cutoff of row k1}, p2[k2] =
// exp(-i phase_coef fy^2); phase_coef = pi * lambda * dz.  The phase is formed and reduced
// mod 2 pi in FP64.
__global__ void prop_table_kernel(float4* p1, float2* p2, const int* cut, int n1, int n2, double dfx64,
                                  double dfy64, double phase_coef, double inv_n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n1 + n2) {
        const bool first = i < n1;
        const int k = first ? fftfreq_int(i, n1) : fftfreq_int(i - n1, n2);
        const double f = (double)k * (first ? dfx64 : dfy64);
        double ph = phase_coef * f * f;
        ph = fma(-TWO_PI, rint(ph * INV_TWO_PI), ph);
        float s, c;
        sincosf((float)ph, &s, &c);
        if (first) {
            const float sc = (float)inv_n;
            p1[i] = make_float4(c * sc, -s * sc, __int_as_float(cut[i]), 0.f);
        } else {
            p2[i - n1] = make_float2(c, -s);
        }
    }
}

int prop_tables(float4* p1, float2* p2, const int* cut, int n1, int n2, double dfx64, double dfy64,
                double phase_coef, double inv_n, cudaStream_t st) {
    prop_table_kernel<<<ceil_div(n1 + n2, 256), 256, 0, st>>>(p1, p2, cut, n1, n2, dfx64, dfy64, phase_coef,
                                                              inv_n);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

}  // namespace emsim_gb300

extern "C" const char* emsim_gb300_last_error(void) { return emsim_gb300::get_error(); }

extern "C" int emsim_gb300_check_device_error(int* code) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(code != nullptr, EMSIM_GB300_ERR_INVALID, "check_device_error: null output");
    *code = 0;
    int dev = 0;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_TRY(ensure_twiddles(dev));
    EMSIM_CHECK_CUDA(cudaDeviceSynchronize());
    volatile int* w = g_err_host + dev;
    *code = *w;
    *w = 0;
    return EMSIM_GB300_OK;
}

extern "C" int emsim_gb300_peek_device_error(int* code) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(code != nullptr, EMSIM_GB300_ERR_INVALID, "peek_device_error: null output");
    *code = 0;
    if (!g_err_host) return EMSIM_GB300_OK;  // no kernel of this library has run yet
    int dev = 0;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_REQUIRE(dev >= 0 && dev < 64, EMSIM_GB300_ERR_UNSUPPORTED, "device index above 63");
    *code = *(volatile int*)(g_err_host + dev);
    return EMSIM_GB300_OK;
}

extern "C" int emsim_gb300_set_wait_limit_ns(unsigned long long ns) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(ns >= tma::MIN_WAIT_LIMIT_NS, EMSIM_GB300_ERR_INVALID,
                  "set_wait_limit_ns: the limit must be at least 1 ms (1000000 ns)");
    g_wait_limit_ns.store(ns, std::memory_order_relaxed);
    return EMSIM_GB300_OK;
}

extern "C" unsigned long long emsim_gb300_get_wait_limit_ns(void) { return emsim_gb300::wait_limit_ns(); }

namespace emsim_gb300 {
// One CTA waits on an mbarrier that nothing arrives at (no copy is issued, so nothing is
// in flight): the bounded wait gives up after limit_ns and the kernel records
// DEV_MBAR_TIMEOUT in the error word, exactly as a pipelined pass does when a tile copy
// never lands.
__global__ void wait_timeout_probe_kernel(int* err, unsigned long long limit_ns, int* result) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tma::mbar_init(&bar, 1);
        tma::fence_mbar_init();
    }
    __syncthreads();
    const bool ok = tma::mbar_wait(&bar, 0, limit_ns);
    if (threadIdx.x == 0) {
        if (!ok) tma::record_error(err, tma::DEV_MBAR_TIMEOUT);
        *result = ok ? 1 : 0;
    }
}
}  // namespace emsim_gb300

extern "C" int emsim_gb300_wait_timeout_probe(unsigned long long limit_ns, int* completed, void* stream) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(completed != nullptr, EMSIM_GB300_ERR_INVALID, "wait_timeout_probe: null output");
    EMSIM_REQUIRE(limit_ns >= 1000ull && limit_ns <= tma::DEFAULT_WAIT_LIMIT_NS, EMSIM_GB300_ERR_INVALID,
                  "wait_timeout_probe: limit must be in [1 us, 2 s]");
    int dev = 0;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_TRY(ensure_twiddles(dev));
    cudaStream_t st = (cudaStream_t)stream;
    wait_timeout_probe_kernel<<<1, 32, 0, st>>>(error_word(), limit_ns, completed);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}
extern "C" int emsim_gb300_abi_version(void) { return EMSIM_GB300_ABI_VERSION; }

extern "C" int emsim_gb300_set_pass_tuning(int n, int row_tma, int row_rows, int col_tma, int col_cols) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(fast_len(n), EMSIM_GB300_ERR_INVALID, "set_pass_tuning: n must be a power of two in [8, 4096]");
    if (row_tma == -2) {  // the built-in setting
        std::lock_guard<std::mutex> lk(g_tuning_mu);
        tuning_table()[log2_fast(n)] = default_tuning(n);
        return EMSIM_GB300_OK;
    }
    EMSIM_REQUIRE(row_tma >= -1 && row_tma <= 2 && col_tma >= -1 && col_tma <= 2 && row_rows >= 0 && col_cols >= 0,
                  EMSIM_GB300_ERR_INVALID,
                  "set_pass_tuning: row and column kernels in {-1, 0, 1, 2 (16 values per thread, lengths 256..4096)}, "
                  "tiles >= 0 (row_tma -2: the built-in setting)");
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    PassTuning& t = tuning_table()[log2_fast(n)];
    t.row_tma = row_tma == 1 ? -1 : row_tma;
    t.row_rows = row_rows;
    t.col_tma = col_tma == 1 ? -1 : col_tma;
    t.col_cols = col_cols;
    return EMSIM_GB300_OK;
}

extern "C" int emsim_gb300_get_pass_tuning(int n, int* out) {
    using namespace emsim_gb300;
    EMSIM_REQUIRE(fast_len(n) && out, EMSIM_GB300_ERR_INVALID, "get_pass_tuning: bad arguments");
    const PassTuning t = pass_tuning(n);
    out[0] = t.row_tma;
    out[1] = t.row_rows;
    out[2] = t.col_tma;
    out[3] = t.col_cols;
    // the tiles the launchers would use without hints (TMA row, simple row, TMA column, simple column)
    out[4] = n >= 16 ? (n / 8 > 256 ? n / 8 : 256) / (n / 8) : 0;
    out[5] = row_threads(n) / (n / 8);
    out[6] = col_tma_B(n, n);
    out[7] = col_B_for(n, n);
    return EMSIM_GB300_OK;
}
