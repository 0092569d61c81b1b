// Wave-propagator plan and its C-ABI entry points (include/emsim_gb300.h).
//
// Replaces emsim::cuda::WavePropagator (emsim/backend/cuda_ext/src/WavePropagator.cu and
// WavePropagator_kernel.cu).  The reference runs four launches per slice (transmit,
// cuFFT forward, propagate, cuFFT inverse); here a slice step is one fused row pass and
// one fused column pass, and the plane wave, exit wave, lens and |psi|^2 are folded into
// the neighbouring passes when the whole image is formed in one call.
#include <cmath>
#include <cstring>
#include <vector>

#include "wave_plan.h"

using namespace emsim_gb300;

namespace emsim_gb300 {

// Reference mask f2 <= filter2 with f2 = fl(fl(fx^2) + fl(fy^2)), fx = fl(k1 * dfx),
// evaluated in float32 (this translation unit is compiled with -ffp-contract=off); for
// fixed k1 it is monotone in |k2|, so one cutoff per row describes the whole disc.
void bandlimit_cutoffs(int n1, int n2, float dfx, float dfy, float filter2, int* cut) {
    for (int i = 0; i < n1; ++i) {
        const float fx = (float)fftfreq_int(i, n1) * dfx;
        const float fx2 = fx * fx;
        int c = -1;
        for (int m = 0; m <= n2 / 2; ++m) {
            const float fy = (float)m * dfy;
            const float fy2 = fy * fy;
            const float f2 = fx2 + fy2;
            if (f2 <= filter2) c = m;
            else break;
        }
        cut[i] = c;
    }
}

int check_device(const emsim_gb300_wave_plan* p) {
    EMSIM_REQUIRE(p != nullptr, EMSIM_GB300_ERR_INVALID, "null wave plan");
    int dev = -1;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_REQUIRE(dev == p->device, EMSIM_GB300_ERR_DEVICE, "wave plan used on a device other than its own");
    return EMSIM_GB300_OK;
}

// FP64 twiddle table exp(-2 pi i m / n) for the generic DFT.
static int make_tw(int n, float2** out) {
    std::vector<float2> h(n);
    for (int m = 0; m < n; ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)n;
        h[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    EMSIM_CHECK_CUDA(cudaMalloc((void**)out, sizeof(float2) * n));
    EMSIM_CHECK_CUDA(cudaMemcpy(*out, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    return EMSIM_GB300_OK;
}

// Propagator tables for dz: p1 (n1, 1/N folded in) then p2 (n2).  Tables are computed on
// the caller's stream the first time a dz is seen and kept, with an event recorded after
// them: a later caller (any stream) waits for that event, so concurrent calls on several
// streams of one plan read finished tables.  With more than PROP_SLOTS distinct dz values
// the oldest slot is rewritten (calls with different dz on different streams of one plan
// must then be ordered by the caller).
size_t prop_slot_bytes(const emsim_gb300_wave_plan* p) {
    return (size_t)p->n1 * sizeof(float4) + (size_t)p->n2 * sizeof(float2);
}

int get_prop(emsim_gb300_wave_plan* p, double dz, cudaStream_t st, const float4** p1, const float2** p2) {
    std::lock_guard<std::mutex> lk(p->mu);
    const size_t sb = prop_slot_bytes(p);
    // inside a CUDA-graph capture the events are left alone (an event recorded outside
    // the capture cannot be waited on inside it); the graph orders its own nodes
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    EMSIM_CHECK_CUDA(cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    for (int i = 0; i < p->prop_used; ++i) {
        if (p->prop_dz[i] == dz) {
            if (p->prop_ev[i] && !capturing) EMSIM_CHECK_CUDA(cudaStreamWaitEvent(st, p->prop_ev[i], 0));
            *p1 = reinterpret_cast<const float4*>(p->prop + (size_t)i * sb);
            *p2 = reinterpret_cast<const float2*>(*p1 + p->n1);
            return EMSIM_GB300_OK;
        }
    }
    int slot = p->prop_used < PROP_SLOTS ? p->prop_used++ : (p->prop_next++ % PROP_SLOTS);
    float4* t1 = reinterpret_cast<float4*>(p->prop + (size_t)slot * sb);
    float2* t2 = reinterpret_cast<float2*>(t1 + p->n1);
    const double coef = M_PI * p->wave_length * dz;
    EMSIM_TRY(prop_tables(t1, t2, p->cut, p->n1, p->n2, p->dfx64, p->dfy64, coef,
                          1.0 / ((double)p->n1 * (double)p->n2), st));
    if (!capturing) {
        if (!p->prop_ev[slot]) EMSIM_CHECK_CUDA(cudaEventCreateWithFlags(&p->prop_ev[slot], cudaEventDisableTiming));
        EMSIM_CHECK_CUDA(cudaEventRecord(p->prop_ev[slot], st));
    } else if (p->prop_ev[slot]) {
        // the slot's old event no longer describes its tables
        cudaEventDestroy(p->prop_ev[slot]);
        p->prop_ev[slot] = nullptr;
    }
    p->prop_dz[slot] = dz;
    *p1 = t1;
    *p2 = t2;
    return EMSIM_GB300_OK;
}

ColArgs base_col(const emsim_gb300_wave_plan* p, float2* data) {
    ColArgs a;
    a.tw = p->tw;
    a.err = p->err;
    a.data = data;
    a.img_stride = (long long)p->n1 * p->n2;
    a.n_rows = p->n1;
    a.n_cols = p->n2;
    a.dfx = p->dfx;
    a.dfy = p->dfy;
    a.filter2 = p->filter2;
    a.dfx64 = p->dfx64;
    a.dfy64 = p->dfy64;
    // propagation keeps |k2| <= cut_max only: columns 0..cut_max and n2-cut_max..n2-1
    a.live_lo = p->cut_max + 1;
    a.live_hi = p->cut_max > 0 ? p->cut_max : 0;
    return a;
}

RowArgs base_row(const emsim_gb300_wave_plan* p) {
    RowArgs a;
    a.tw = p->tw;
    a.err = p->err;
    const long long npix = (long long)p->n1 * p->n2;
    a.in_img_stride = npix;
    a.out_img_stride = npix;
    a.out_int_img_stride = npix;
    a.sigma = p->sigma;
    a.sigma_pi = p->sigma_pi;
    a.n_rows = p->n1;
    return a;
}

// lens transfer constants (FP64): chi = f2 * (c1 * f2 - c2), c1 = pi/2 Cs lambda^3,
// c2 = pi lambda defocus (WavePropagator.cpp:107-109 in float32 there)
void set_lens(const emsim_gb300_wave_plan* p, ColArgs& a, double cs_mm, double aperture, float scale) {
    const double lam = p->wave_length;
    a.c1 = 0.5 * M_PI * cs_mm * 1e7 * lam * lam * lam;
    const float fap = (float)aperture / (float)lam;  // aperture / waveLength in float32
    a.aper2 = fap * fap;
    a.lens_scale = scale;
}

}  // namespace emsim_gb300

namespace {

// ---- the generic (any size) path -------------------------------------------------
int g_fft2(emsim_gb300_wave_plan* p, const float2* in, float2* out, bool inverse, int nb, cudaStream_t st) {
    // forward: rows then columns; inverse: columns then rows (both unnormalised)
    if (!inverse) {
        EMSIM_TRY(generic_dft_rows(in, out, p->n1, p->n2, false, p->tw2, nb, st));
        EMSIM_TRY(generic_dft_cols(out, p->n1, p->n2, false, p->tw1, nb, st));
    } else {
        if (in != out) EMSIM_CHECK_CUDA(cudaMemcpyAsync(out, in, sizeof(float2) * (size_t)nb * p->n1 * p->n2,
                                                        cudaMemcpyDeviceToDevice, st));
        EMSIM_TRY(generic_dft_cols(out, p->n1, p->n2, true, p->tw1, nb, st));
        EMSIM_TRY(generic_dft_rows(out, out, p->n1, p->n2, true, p->tw2, nb, st));
    }
    return EMSIM_GB300_OK;
}

int g_space(emsim_gb300_wave_plan* p, const float2* in, float2* out, double dz, int nb, cudaStream_t st) {
    const float4* p1;
    const float2* p2;
    EMSIM_TRY(get_prop(p, dz, st, &p1, &p2));
    EMSIM_TRY(g_fft2(p, in, out, false, nb, st));
    ColArgs a = base_col(p, out);
    a.p1 = p1;
    a.p2 = p2;
    EMSIM_TRY(ew_propagate(out, a, nb, st));
    return g_fft2(p, out, out, true, nb, st);
}

int g_lens(emsim_gb300_wave_plan* p, const float2* in, float2* out, double cs, const double* defocus, int n_def,
           double aperture, int nb, cudaStream_t st, double es = 0.0) {
    EMSIM_TRY(g_fft2(p, in, out, false, nb, st));
    for (int i0 = 0; i0 < nb; i0 += LENS_MAX) {
        const int cnt = nb - i0 < LENS_MAX ? nb - i0 : LENS_MAX;
        ColArgs a = base_col(p, out + (size_t)i0 * p->n1 * p->n2);
        set_lens(p, a, cs, aperture, 1.0f / (float)((double)p->n1 * p->n2));
        a.es = es;
        a.n_c2 = n_def == 1 ? 1 : cnt;
        for (int j = 0; j < a.n_c2; ++j) a.c2v[j] = M_PI * p->wave_length * defocus[(i0 + j) % n_def];
        EMSIM_TRY(ew_lens(a.data, a, cnt, st));
    }
    return g_fft2(p, out, out, true, nb, st);
}

}  // namespace

extern "C" {

int emsim_gb300_wave_plan_create(int n1, int n2, double d1, double d2, double wave_length,
                                 double relativity_gamma, emsim_gb300_wave_plan** plan) {
    EMSIM_REQUIRE(plan != nullptr, EMSIM_GB300_ERR_INVALID, "null plan output pointer");
    *plan = nullptr;
    EMSIM_REQUIRE(n1 > 0 && n2 > 0, EMSIM_GB300_ERR_INVALID, "wave shape must be positive");
    EMSIM_REQUIRE(d1 > 0 && d2 > 0 && wave_length > 0, EMSIM_GB300_ERR_INVALID,
                  "pixel size and wave length must be positive");
    EMSIM_REQUIRE(n1 <= 16384 && n2 <= 16384, EMSIM_GB300_ERR_UNSUPPORTED, "wave side above 16384");
    auto* p = new emsim_gb300_wave_plan();
    p->n1 = n1;
    p->n2 = n2;
    p->d1 = d1;
    p->d2 = d2;
    p->wave_length = wave_length;
    p->gamma = relativity_gamma;
    p->sigma = (float)(wave_length * relativity_gamma);
    p->sigma_pi = (float)(wave_length * relativity_gamma / M_PI);
    const float d1f = (float)d1, d2f = (float)d2;
    p->dfx = 1.0f / d1f / (float)n1;
    p->dfy = 1.0f / d2f / (float)n2;
    const float fmax = 0.5f / (d1f >= d2f ? d1f : d2f);
    const float filt = 0.6667f * fmax;
    p->filter2 = filt * filt;
    p->dfx64 = 1.0 / (d1 * n1);
    p->dfy64 = 1.0 / (d2 * n2);
    p->fast = fast_len(n1) && fast_len(n2);
    int st = EMSIM_GB300_OK;
    auto fail = [&](int code) {
        if (p->tw1) cudaFree(p->tw1);
        if (p->tw2) cudaFree(p->tw2);
        if (p->prop) cudaFree(p->prop);
        if (p->cut) cudaFree(p->cut);
        delete p;
        return code;
    };
    if (cudaGetDevice(&p->device) != cudaSuccess) {
        set_error("cudaGetDevice failed");
        return fail(EMSIM_GB300_ERR_CUDA);
    }
    if ((st = ensure_twiddles(p->device)) != EMSIM_GB300_OK) return fail(st);
    p->tw = twiddle_table();
    p->err = error_word();
    if (!p->fast) {
        if ((st = make_tw(n1, &p->tw1)) != EMSIM_GB300_OK) return fail(st);
        if ((st = make_tw(n2, &p->tw2)) != EMSIM_GB300_OK) return fail(st);
        // chirp tables of the Bluestein line transforms, built here rather than on first use
        if ((st = bluestein_prepare(n1)) != EMSIM_GB300_OK) return fail(st);
        if ((st = bluestein_prepare(n2)) != EMSIM_GB300_OK) return fail(st);
    }
    if (cudaMalloc((void**)&p->prop, prop_slot_bytes(p) * PROP_SLOTS) != cudaSuccess ||
        cudaMalloc((void**)&p->cut, sizeof(int) * n1) != cudaSuccess) {
        set_error("cudaMalloc of propagator tables failed");
        return fail(EMSIM_GB300_ERR_CUDA);
    }
    {
        std::vector<int> cut(n1);
        bandlimit_cutoffs(n1, n2, p->dfx, p->dfy, p->filter2, cut.data());
        for (int i = 0; i < n1; ++i) p->cut_max = cut[i] > p->cut_max ? cut[i] : p->cut_max;
        if (cudaMemcpy(p->cut, cut.data(), sizeof(int) * n1, cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("upload of band-limit cutoffs failed");
            return fail(EMSIM_GB300_ERR_CUDA);
        }
    }
    *plan = p;
    return EMSIM_GB300_OK;
}

int emsim_gb300_wave_plan_destroy(emsim_gb300_wave_plan* p) {
    if (!p) return EMSIM_GB300_OK;
    for (cudaEvent_t& e : p->prop_ev)
        if (e) cudaEventDestroy(e);
    cudaFree(p->tw1);
    cudaFree(p->tw2);
    cudaFree(p->prop);
    cudaFree(p->cut);
    delete p;
    return EMSIM_GB300_OK;
}

int emsim_gb300_init_wave(emsim_gb300_wave_plan* p, double dose, void* wave_out, int nb, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(wave_out && nb >= 1, EMSIM_GB300_ERR_INVALID, "init_wave: bad output or batch");
    // sqrt(dose * d1 * d2) in FP64, rounded once to complex64 (wave_propagator_base.py:25-29)
    const float amp = (float)std::sqrt(dose * p->d1 * p->d2);
    return ew_fill((float2*)wave_out, (long long)nb * p->n1 * p->n2, make_float2(amp, 0.f), (cudaStream_t)stream);
}

int emsim_gb300_slice_transmit(emsim_gb300_wave_plan* p, const void* wave, const float* slice,
                               long long slice_stride, void* wave_out, int nb, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(wave && slice && wave_out && nb >= 1, EMSIM_GB300_ERR_INVALID, "slice_transmit: bad arguments");
    const long long npix = (long long)p->n1 * p->n2;
    return ew_transmit((const float2*)wave, slice, (float2*)wave_out, npix, p->sigma_pi, nb, npix, slice_stride, npix,
                       (cudaStream_t)stream);
}

int emsim_gb300_space_propagate(emsim_gb300_wave_plan* p, const void* wave, double dz, void* wave_out, int nb,
                                void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(wave && wave_out && nb >= 1, EMSIM_GB300_ERR_INVALID, "space_propagate: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    float2* out = (float2*)wave_out;
    if (!p->fast) return g_space(p, (const float2*)wave, out, dz, nb, st);
    const float4* p1;
    const float2* p2;
    EMSIM_TRY(get_prop(p, dz, st, &p1, &p2));
    RowArgs r = base_row(p);
    r.in = (const float2*)wave;
    r.out = out;
    EMSIM_TRY(launch_row(p->n2, ROW_FFT, r, nb, st));
    ColArgs c = base_col(p, out);
    c.p1 = p1;
    c.p2 = p2;
    EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, c, nb, st));
    r.in = out;
    return launch_row(p->n2, ROW_IFFT, r, nb, st);
}

int emsim_gb300_singleslice_propagate(emsim_gb300_wave_plan* p, const void* wave, const float* slice,
                                      long long slice_stride, double dz, void* wave_out, int nb, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(wave && slice && wave_out && nb >= 1, EMSIM_GB300_ERR_INVALID,
                  "singleslice_propagate: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    float2* out = (float2*)wave_out;
    const long long npix = (long long)p->n1 * p->n2;
    if (!p->fast) {
        EMSIM_TRY(ew_transmit((const float2*)wave, slice, out, npix, p->sigma_pi, nb, npix, slice_stride, npix, st));
        return g_space(p, out, out, dz, nb, st);
    }
    const float4* p1;
    const float2* p2;
    EMSIM_TRY(get_prop(p, dz, st, &p1, &p2));
    RowArgs r = base_row(p);
    r.in = (const float2*)wave;
    r.out = out;
    r.slice = slice;
    r.slice_img_stride = slice_stride;
    EMSIM_TRY(launch_row(p->n2, ROW_TRANSMIT | ROW_FFT, r, nb, st));
    ColArgs c = base_col(p, out);
    c.p1 = p1;
    c.p2 = p2;
    EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, c, nb, st));
    r.in = out;
    return launch_row(p->n2, ROW_IFFT, r, nb, st);
}

}  // extern "C"

namespace {

// Multislice steps on the fast path.  On return `work` holds the "row-inverse pending"
// state X of the last step (psi_exit = IFFT_rows(X), unnormalised).  const_in: start
// from the plane wave const_val instead of reading `in`.
int fast_steps(emsim_gb300_wave_plan* p, const float2* in, bool const_in, float2 const_val, const float* slices,
               int n_slices, long long slices_stride, double dz, float2* work, int nb, cudaStream_t st) {
    const float4* p1;
    const float2* p2;
    EMSIM_TRY(get_prop(p, dz, st, &p1, &p2));
    const long long npix = (long long)p->n1 * p->n2;
    RowArgs r = base_row(p);
    r.out = work;
    r.slice_img_stride = slices_stride;
    ColArgs c = base_col(p, work);
    c.p1 = p1;
    c.p2 = p2;
    for (int s = 0; s < n_slices; ++s) {
        r.slice = slices + (long long)s * npix;
        int ops;
        if (s == 0) {
            ops = const_in ? (ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT) : (ROW_TRANSMIT | ROW_FFT);
            r.in = in;
            r.const_val = const_val;
        } else {
            ops = ROW_IFFT | ROW_TRANSMIT | ROW_FFT;
            r.in = work;
        }
        EMSIM_TRY(launch_row(p->n2, ops, r, nb, st));
        EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, c, nb, st));
    }
    return EMSIM_GB300_OK;
}

}  // namespace

extern "C" {

int emsim_gb300_multislice_propagate(emsim_gb300_wave_plan* p, const void* wave, const float* slices,
                                     int n_slices, long long slices_stride, double dz, void* wave_out, int nb,
                                     void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(wave && wave_out && nb >= 1 && n_slices >= 0 && (slices || n_slices == 0),
                  EMSIM_GB300_ERR_INVALID, "multislice_propagate: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    float2* out = (float2*)wave_out;
    const long long npix = (long long)p->n1 * p->n2;
    if (n_slices == 0) {
        if (wave != wave_out)
            EMSIM_CHECK_CUDA(cudaMemcpyAsync(out, wave, sizeof(float2) * npix * nb, cudaMemcpyDeviceToDevice, st));
        return EMSIM_GB300_OK;
    }
    if (!p->fast) {
        const float2* cur = (const float2*)wave;
        for (int s = 0; s < n_slices; ++s) {
            EMSIM_TRY(ew_transmit(cur, slices + (long long)s * npix, out, npix, p->sigma_pi, nb, npix, slices_stride,
                                  npix, st));
            EMSIM_TRY(g_space(p, out, out, dz, nb, st));
            cur = out;
        }
        return EMSIM_GB300_OK;
    }
    EMSIM_TRY(fast_steps(p, (const float2*)wave, false, make_float2(0.f, 0.f), slices, n_slices, slices_stride, dz,
                         out, nb, st));
    RowArgs r = base_row(p);
    r.in = out;
    r.out = out;
    return launch_row(p->n2, ROW_IFFT, r, nb, st);
}

int emsim_gb300_lens_propagate(emsim_gb300_wave_plan* p, const void* wave, double cs_mm, double defocus,
                               double aperture, void* wave_out, int nb, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(wave && wave_out && nb >= 1, EMSIM_GB300_ERR_INVALID, "lens_propagate: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    float2* out = (float2*)wave_out;
    if (!p->fast) return g_lens(p, (const float2*)wave, out, cs_mm, &defocus, 1, aperture, nb, st);
    RowArgs r = base_row(p);
    r.in = (const float2*)wave;
    r.out = out;
    EMSIM_TRY(launch_row(p->n2, ROW_FFT, r, nb, st));
    ColArgs c = base_col(p, out);
    set_lens(p, c, cs_mm, aperture, 1.0f / (float)((double)p->n1 * p->n2));
    c.n_c2 = 1;
    c.c2v[0] = M_PI * p->wave_length * defocus;
    EMSIM_TRY(launch_col(p->n1, COL_LENS, c, nb, st));
    r.in = out;
    return launch_row(p->n2, ROW_IFFT, r, nb, st);
}

size_t emsim_gb300_lens_incoherent_workspace_size(const emsim_gb300_wave_plan* p, int nb) {
    if (!p || nb < 1) return 0;
    const size_t npix = (size_t)p->n1 * p->n2 * (size_t)nb;
    // fast path: row spectrum X and a working copy (complex), one intensity (float)
    return npix * (2 * sizeof(float2) + sizeof(float)) + 256;
}

int emsim_gb300_lens_intensity_incoherent(emsim_gb300_wave_plan* p, const void* exit_wave, int nb, double cs_mm,
                                          const double* defocus, const double* weights, int n_defocus,
                                          double illumination_angle, double aperture, float* image_out, void* work,
                                          size_t work_bytes, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(exit_wave && image_out && work && defocus && weights && n_defocus >= 1 && nb >= 1 &&
                      illumination_angle >= 0.0,
                  EMSIM_GB300_ERR_INVALID, "lens_intensity_incoherent: bad arguments");
    EMSIM_REQUIRE(work_bytes >= emsim_gb300_lens_incoherent_workspace_size(p, nb), EMSIM_GB300_ERR_INVALID,
                  "lens_intensity_incoherent: workspace smaller than lens_incoherent_workspace_size");
    cudaStream_t st = (cudaStream_t)stream;
    const long long npix = (long long)p->n1 * p->n2;
    const long long n_all = npix * nb;
    float2* x = reinterpret_cast<float2*>(work);
    float2* y = x + n_all;
    float* ik = reinterpret_cast<float*>(y + n_all);
    const double es = (illumination_angle / p->wave_length) * (illumination_angle / p->wave_length);
    EMSIM_CHECK_CUDA(cudaMemsetAsync(image_out, 0, sizeof(float) * (size_t)n_all, st));
    RowArgs r = base_row(p);
    if (p->fast) {
        r.in = (const float2*)exit_wave;
        r.out = x;
        EMSIM_TRY(launch_row(p->n2, ROW_FFT, r, nb, st));
    }
    for (int k = 0; k < n_defocus; ++k) {
        if (p->fast) {
            EMSIM_CHECK_CUDA(cudaMemcpyAsync(y, x, sizeof(float2) * (size_t)n_all, cudaMemcpyDeviceToDevice, st));
            ColArgs c = base_col(p, y);
            set_lens(p, c, cs_mm, aperture, 1.0f / (float)npix);
            c.es = es;
            c.n_c2 = 1;
            c.c2v[0] = M_PI * p->wave_length * defocus[k];
            EMSIM_TRY(launch_col(p->n1, COL_LENS, c, nb, st));
            r.in = y;
            r.out_int = ik;
            EMSIM_TRY(launch_row(p->n2, ROW_IFFT | ROW_OUT_INTENSITY, r, nb, st));
        } else {
            EMSIM_TRY(g_lens(p, (const float2*)exit_wave, y, cs_mm, defocus + k, 1, aperture, nb, st, es));
            EMSIM_TRY(ew_intensity(y, ik, n_all, st));
        }
        EMSIM_TRY(ew_axpy(image_out, ik, (float)weights[k], n_all, st));
    }
    return EMSIM_GB300_OK;
}

int emsim_gb300_intensity(const void* wave, float* out, long long n, void* stream) {
    EMSIM_REQUIRE(wave && out && n >= 0, EMSIM_GB300_ERR_INVALID, "intensity: bad arguments");
    if (n == 0) return EMSIM_GB300_OK;
    return ew_intensity((const float2*)wave, out, n, (cudaStream_t)stream);
}

int emsim_gb300_multislice_image(emsim_gb300_wave_plan* p, const float* slices, int n_slices,
                                 long long slices_stride, double dz, double dose, double cs_mm,
                                 const double* defocus, int n_defocus, double aperture, float* image_out,
                                 void* wave_work, void* exit_wave_out, int nb, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(image_out && wave_work && nb >= 1 && n_slices >= 0 && (slices || n_slices == 0) && defocus &&
                      n_defocus >= 1,
                  EMSIM_GB300_ERR_INVALID, "multislice_image: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    float2* work = (float2*)wave_work;
    const long long npix = (long long)p->n1 * p->n2;
    const float amp = (float)std::sqrt(dose * p->d1 * p->d2);
    if (!p->fast || n_slices == 0) {
        EMSIM_TRY(ew_fill(work, npix * nb, make_float2(amp, 0.f), st));
        EMSIM_TRY(emsim_gb300_multislice_propagate(p, work, slices, n_slices, slices_stride, dz, work, nb, stream));
        if (exit_wave_out)
            EMSIM_CHECK_CUDA(
                cudaMemcpyAsync(exit_wave_out, work, sizeof(float2) * npix * nb, cudaMemcpyDeviceToDevice, st));
        if (!p->fast) {
            EMSIM_TRY(g_lens(p, work, work, cs_mm, defocus, n_defocus, aperture, nb, st));
        } else {
            RowArgs r = base_row(p);
            r.in = work;
            r.out = work;
            EMSIM_TRY(launch_row(p->n2, ROW_FFT, r, nb, st));
            for (int i0 = 0; i0 < nb; i0 += LENS_MAX) {
                const int cnt = nb - i0 < LENS_MAX ? nb - i0 : LENS_MAX;
                ColArgs c = base_col(p, work + i0 * npix);
                set_lens(p, c, cs_mm, aperture, 1.0f / (float)npix);
                c.n_c2 = n_defocus == 1 ? 1 : cnt;
                for (int j = 0; j < c.n_c2; ++j) c.c2v[j] = M_PI * p->wave_length * defocus[(i0 + j) % n_defocus];
                EMSIM_TRY(launch_col(p->n1, COL_LENS, c, cnt, st));
            }
            EMSIM_TRY(launch_row(p->n2, ROW_IFFT, r, nb, st));
        }
        return ew_intensity(work, image_out, npix * nb, st);
    }
    EMSIM_TRY(fast_steps(p, nullptr, true, make_float2(amp, 0.f), slices, n_slices, slices_stride, dz, work, nb, st));
    RowArgs r = base_row(p);
    if (exit_wave_out) {
        r.in = work;
        r.out = (float2*)exit_wave_out;
        EMSIM_TRY(launch_row(p->n2, ROW_IFFT, r, nb, st));
    }
    // FFT2(psi_exit) = n2 * FFT_cols(X): the lens acts on X directly with 1/n1 instead of 1/N
    for (int i0 = 0; i0 < nb; i0 += LENS_MAX) {
        const int cnt = nb - i0 < LENS_MAX ? nb - i0 : LENS_MAX;
        ColArgs c = base_col(p, work + i0 * npix);
        set_lens(p, c, cs_mm, aperture, 1.0f / (float)p->n1);
        c.n_c2 = n_defocus == 1 ? 1 : cnt;
        for (int j = 0; j < c.n_c2; ++j) c.c2v[j] = M_PI * p->wave_length * defocus[(i0 + j) % n_defocus];
        EMSIM_TRY(launch_col(p->n1, COL_LENS, c, cnt, st));
    }
    r.in = work;
    r.out_int = image_out;
    return launch_row(p->n2, ROW_IFFT | ROW_OUT_INTENSITY, r, nb, st);
}

int emsim_gb300_multislice_image_ragged(emsim_gb300_wave_plan* p, const float* slices, long long slices_stride,
                                        const int32_t* n_slices, double dz, double dose, double cs_mm,
                                        const double* defocus, int n_defocus, double aperture, float* image_out,
                                        void* wave_work, int nb, void* stream) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(p->fast, EMSIM_GB300_ERR_UNSUPPORTED,
                  "multislice_image_ragged: wave sides must be powers of two between 8 and 4096");
    EMSIM_REQUIRE(slices && n_slices && image_out && wave_work && defocus && n_defocus >= 1 && nb >= 1,
                  EMSIM_GB300_ERR_INVALID, "multislice_image_ragged: bad arguments");
    const long long npix = (long long)p->n1 * p->n2;
    for (int i = 0; i < nb; ++i) {
        EMSIM_REQUIRE(n_slices[i] >= 1 && (i == 0 || n_slices[i] <= n_slices[i - 1]), EMSIM_GB300_ERR_INVALID,
                      "multislice_image_ragged: slice counts must be >= 1 and non-increasing");
    }
    EMSIM_REQUIRE(nb == 1 || slices_stride >= (long long)n_slices[0] * npix, EMSIM_GB300_ERR_INVALID,
                  "multislice_image_ragged: slices_stride below the longest stack");
    cudaStream_t st = (cudaStream_t)stream;
    float2* work = (float2*)wave_work;
    const float4* p1;
    const float2* p2;
    EMSIM_TRY(get_prop(p, dz, st, &p1, &p2));
    RowArgs r = base_row(p);
    r.out = work;
    r.slice_img_stride = slices_stride;
    r.const_val = make_float2((float)std::sqrt(dose * p->d1 * p->d2), 0.f);
    ColArgs c = base_col(p, work);
    c.p1 = p1;
    c.p2 = p2;
    int active = nb;  // images with a slice s form a prefix of the batch
    for (int s = 0; s < n_slices[0]; ++s) {
        while (active > 0 && n_slices[active - 1] <= s) --active;
        r.slice = slices + (long long)s * npix;
        r.in = work;
        const int ops = s == 0 ? (ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT) : (ROW_IFFT | ROW_TRANSMIT | ROW_FFT);
        EMSIM_TRY(launch_row(p->n2, ops, r, active, st));
        EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, c, active, st));
    }
    for (int i0 = 0; i0 < nb; i0 += LENS_MAX) {
        const int cnt = nb - i0 < LENS_MAX ? nb - i0 : LENS_MAX;
        ColArgs cl = base_col(p, work + i0 * npix);
        set_lens(p, cl, cs_mm, aperture, 1.0f / (float)p->n1);
        cl.n_c2 = n_defocus == 1 ? 1 : cnt;
        for (int j = 0; j < cl.n_c2; ++j) cl.c2v[j] = M_PI * p->wave_length * defocus[(i0 + j) % n_defocus];
        EMSIM_TRY(launch_col(p->n1, COL_LENS, cl, cnt, st));
    }
    RowArgs ri = base_row(p);
    ri.in = work;
    ri.out_int = image_out;
    return launch_row(p->n2, ROW_IFFT | ROW_OUT_INTENSITY, ri, nb, st);
}

}  // extern "C"
