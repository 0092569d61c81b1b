// Checkpointed forward and adjoint of the fused image: I = |L P t_{S-1} ... P t_0 psi_0|^2.
//
// emsim itself has no derivative of the multislice image; this is the differentiable
// form of emsim_gb300_multislice_image (pipe.py:46-55, 79-84 forward).  Notation:
//   psi_0 = sqrt(dose d1 d2)                 plane wave
//   phi_s = psi_s * t_s,  t_s = exp(i sigma V_s)   transmit (WavePropagator_kernel.cu:12-43)
//   psi_{s+1} = P phi_s                       Fresnel step with the 2/3 band limit
//   u = L psi_S,  I = |u|^2                   lens / CTF with aperture
// For a real loss with g = dLoss/dI:
//   lambda_u = g u,  lambda_{psi_S} = L^H lambda_u,
//   mu_s = P^H lambda_{psi_{s+1}},  lambda_{psi_s} = conj(t_s) mu_s,
//   dLoss/dV_s = 2 sigma Im(mu_s conj(phi_s)).
// P and L are diagonal in Fourier space, so P^H is the step with -dz (conjugate phase,
// same real band-limit mask) and L^H the lens with (-Cs, -defocus) (conjugate chi, same
// real aperture).  Both sweeps use the forward's two fused passes in the same
// "row-inverse pending" form; the adjoint row pass adds the gradient (ROW_GRAD) and the
// conjugate transmit (sigma -> -sigma), the recompute row pass stores phi_s
// (ROW_STORE_PHI).
//
// Memory: the forward keeps the row-pending state X_s of every K-th step (K = `every`,
// about sqrt(S) gives O(sqrt(S)) waves); the adjoint walks the segments backwards,
// recomputes the K transmitted waves phi_s of one segment from its checkpoint, then runs
// the K adjoint steps of that segment.
#include <cmath>
#include <cstdint>

#include "wave_plan.h"

using namespace emsim_gb300;

namespace {

constexpr size_t ALIGN = 256;

size_t align_up(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

// lambda_u = g * u (complex times real), n elements
__global__ void lambda_init_kernel(const float2* __restrict__ u, const float* __restrict__ g, float2* lam,
                                   long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 a = u[i];
        const float w = g[i];
        lam[i] = make_float2(a.x * w, a.y * w);
    }
}

// out[p] = sum over images i = 0..nb-1, in that order, of part[i * npix + p]
__global__ void reduce_images_kernel(const float* __restrict__ part, float* out, long long npix, int nb) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int i = 0; i < nb; ++i) s += part[(long long)i * npix + p];
        out[p] = s;
    }
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 152 * 16 ? (g < 1 ? 1 : g) : 152 * 16);
}

int n_checkpoints(int n_slices, int every) { return (n_slices + every - 1) / every - 1; }

struct AdjointWorkspace {
    float2* lam = nullptr;   // adjoint state, nb images
    float2* seg = nullptr;   // recompute state, nb images
    float2* phi = nullptr;   // K x nb transmitted waves of one segment
    float* part = nullptr;   // per-image gradients of one slice (shared slices, nb > 1)
    size_t bytes = 0;
};

AdjointWorkspace layout(const emsim_gb300_wave_plan* p, int n_slices, int every, int nb, long long slices_stride,
                        char* base) {
    AdjointWorkspace w;
    const size_t npix = (size_t)p->n1 * p->n2;
    const size_t wave = align_up(sizeof(float2) * npix * nb);
    const int k = every < n_slices ? every : n_slices;
    const size_t part = (slices_stride == 0 && nb > 1) ? align_up(sizeof(float) * npix * nb) : 0;
    w.bytes = wave * (2 + (size_t)k) + part;
    if (base != nullptr) {
        w.lam = (float2*)base;
        w.seg = (float2*)(base + wave);
        w.phi = (float2*)(base + 2 * wave);
        if (part) w.part = (float*)(base + wave * (2 + (size_t)k));
    }
    return w;
}

int check_args(const emsim_gb300_wave_plan* p, int n_slices, long long slices_stride, int every, int nb,
               const double* defocus, int n_defocus) {
    EMSIM_TRY(check_device(p));
    EMSIM_REQUIRE(p->fast, EMSIM_GB300_ERR_UNSUPPORTED,
                  "adjoint: wave sides must be powers of two between 8 and 4096");
    EMSIM_REQUIRE(n_slices >= 1 && every >= 1 && nb >= 1 && defocus != nullptr && n_defocus >= 1,
                  EMSIM_GB300_ERR_INVALID, "adjoint: need n_slices >= 1, every >= 1, nb >= 1 and a defocus list");
    const long long npix = (long long)p->n1 * p->n2;
    EMSIM_REQUIRE(slices_stride == 0 || slices_stride >= (long long)n_slices * npix, EMSIM_GB300_ERR_INVALID,
                  "adjoint: slices_stride must be 0 (shared) or at least n_slices * n1 * n2");
    return EMSIM_GB300_OK;
}

// lens column pass over nb images (defocus of image i = defocus[i % n_defocus]); adjoint
// negates Cs and the defocus (conjugate transfer function)
int lens_cols(emsim_gb300_wave_plan* p, float2* data, double cs_mm, const double* defocus, int n_defocus,
              double aperture, bool adjoint, int nb, cudaStream_t st) {
    const long long npix = (long long)p->n1 * p->n2;
    const double sgn = adjoint ? -1.0 : 1.0;
    for (int i0 = 0; i0 < nb; i0 += LENS_MAX) {
        const int cnt = nb - i0 < LENS_MAX ? nb - i0 : LENS_MAX;
        ColArgs c = base_col(p, data + (long long)i0 * npix);
        // FFT2(IFFT_rows(X)) = n2 FFT_cols(X): acting on X the lens scale is 1/n1
        set_lens(p, c, cs_mm, aperture, 1.0f / (float)p->n1);
        c.c1 *= sgn;
        c.n_c2 = n_defocus == 1 ? 1 : cnt;
        for (int j = 0; j < c.n_c2; ++j) c.c2v[j] = sgn * M_PI * p->wave_length * defocus[(i0 + j) % n_defocus];
        EMSIM_TRY(launch_col(p->n1, COL_LENS, c, cnt, st));
    }
    return EMSIM_GB300_OK;
}

}  // namespace

extern "C" {

int emsim_gb300_adjoint_checkpoints(int n_slices, int every) {
    if (n_slices < 1 || every < 1) return 0;
    return n_checkpoints(n_slices, every);
}

size_t emsim_gb300_adjoint_workspace_size(emsim_gb300_wave_plan* p, int n_slices, int every, int nb,
                                          long long slices_stride) {
    if (p == nullptr || n_slices < 1 || every < 1 || nb < 1) return 0;
    return layout(p, n_slices, every, nb, slices_stride, nullptr).bytes;
}

int emsim_gb300_multislice_image_ckpt(emsim_gb300_wave_plan* p, const float* slices, int n_slices,
                                      long long slices_stride, double dz, double dose, double cs_mm,
                                      const double* defocus, int n_defocus, double aperture, float* image_out,
                                      void* image_wave_out, void* ckpt, int every, int nb, void* stream) {
    EMSIM_TRY(check_args(p, n_slices, slices_stride, every, nb, defocus, n_defocus));
    const int n_ck = n_checkpoints(n_slices, every);
    EMSIM_REQUIRE(slices && image_out && image_wave_out && (ckpt || n_ck == 0), EMSIM_GB300_ERR_INVALID,
                  "multislice_image_ckpt: null slices, image, image wave or checkpoint buffer");
    cudaStream_t st = (cudaStream_t)stream;
    const long long npix = (long long)p->n1 * p->n2;
    float2* work = (float2*)image_wave_out;
    float2* ck = (float2*)ckpt;
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
    for (int s = 0; s < n_slices; ++s) {
        if (s > 0 && s % every == 0) {
            // X_s: the state the row pass of step s starts from
            EMSIM_CHECK_CUDA(cudaMemcpyAsync(ck + (long long)(s / every - 1) * nb * npix, work,
                                             sizeof(float2) * npix * nb, cudaMemcpyDeviceToDevice, st));
        }
        r.slice = slices + (long long)s * npix;
        r.in = work;
        const int ops = s == 0 ? (ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT) : (ROW_IFFT | ROW_TRANSMIT | ROW_FFT);
        EMSIM_TRY(launch_row(p->n2, ops, r, nb, st));
        EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, c, nb, st));
    }
    EMSIM_TRY(lens_cols(p, work, cs_mm, defocus, n_defocus, aperture, false, nb, st));
    r.in = work;
    EMSIM_TRY(launch_row(p->n2, ROW_IFFT, r, nb, st));
    return ew_intensity(work, image_out, npix * nb, st);
}

int emsim_gb300_multislice_image_adjoint(emsim_gb300_wave_plan* p, const float* slices, int n_slices,
                                         long long slices_stride, double dz, double dose, double cs_mm,
                                         const double* defocus, int n_defocus, double aperture,
                                         const float* grad_image, const void* image_wave, const void* ckpt,
                                         int every, float* grad_slices, void* work, size_t work_bytes, int nb,
                                         void* stream) {
    EMSIM_TRY(check_args(p, n_slices, slices_stride, every, nb, defocus, n_defocus));
    const int n_ck = n_checkpoints(n_slices, every);
    EMSIM_REQUIRE(slices && grad_image && image_wave && grad_slices && work && (ckpt || n_ck == 0),
                  EMSIM_GB300_ERR_INVALID, "multislice_image_adjoint: null argument");
    AdjointWorkspace w = layout(p, n_slices, every, nb, slices_stride, (char*)work);
    EMSIM_REQUIRE(work_bytes >= w.bytes, EMSIM_GB300_ERR_INVALID,
                  "multislice_image_adjoint: workspace smaller than emsim_gb300_adjoint_workspace_size");
    EMSIM_REQUIRE(((uintptr_t)work % ALIGN) == 0, EMSIM_GB300_ERR_INVALID,
                  "multislice_image_adjoint: workspace must be 256-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    const long long npix = (long long)p->n1 * p->n2;
    const long long nwave = npix * nb;
    const float4 *p1f, *p1b;
    const float2 *p2f, *p2b;
    EMSIM_TRY(get_prop(p, dz, st, &p1f, &p2f));
    EMSIM_TRY(get_prop(p, -dz, st, &p1b, &p2b));

    // lambda_u = g u -> FFT rows -> conjugate lens: lam = FFT_rows(lambda_{psi_S})
    lambda_init_kernel<<<grid_for(nwave), 256, 0, st>>>((const float2*)image_wave, grad_image, w.lam, nwave);
    EMSIM_CHECK_LAUNCH();
    RowArgs rb = base_row(p);
    rb.in = w.lam;
    rb.out = w.lam;
    EMSIM_TRY(launch_row(p->n2, ROW_FFT, rb, nb, st));
    EMSIM_TRY(lens_cols(p, w.lam, cs_mm, defocus, n_defocus, aperture, true, nb, st));

    ColArgs cb = base_col(p, w.lam);  // P^H: the step with -dz
    cb.p1 = p1b;
    cb.p2 = p2b;
    rb.slice_img_stride = slices_stride;
    rb.sigma = -p->sigma;  // conj(t_s)
    rb.sigma_pi = -p->sigma_pi;
    rb.sigma_grad = p->sigma;
    rb.phi_img_stride = npix;
    const bool reduce = slices_stride == 0 && nb > 1;

    RowArgs rf = base_row(p);  // recompute of phi_s
    rf.out = w.seg;
    rf.slice_img_stride = slices_stride;
    rf.phi_img_stride = npix;
    rf.const_val = make_float2((float)std::sqrt(dose * p->d1 * p->d2), 0.f);
    ColArgs cf = base_col(p, w.seg);
    cf.p1 = p1f;
    cf.p2 = p2f;

    for (int m = n_ck; m >= 0; --m) {
        const int s0 = m * every;
        const int s1 = (s0 + every < n_slices ? s0 + every : n_slices) - 1;
        for (int s = s0; s <= s1; ++s) {
            rf.slice = slices + (long long)s * npix;
            rf.phi = w.phi + (long long)(s - s0) * nwave;
            int ops = ROW_IFFT | ROW_TRANSMIT | ROW_FFT | ROW_STORE_PHI;
            if (s == 0) {
                ops = ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT | ROW_STORE_PHI;
            } else if (s == s0) {
                rf.in = (const float2*)ckpt + (long long)(m - 1) * nwave;
            } else {
                rf.in = w.seg;
            }
            EMSIM_TRY(launch_row(p->n2, ops, rf, nb, st));
            if (s < s1) EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, cf, nb, st));
        }
        for (int s = s1; s >= s0; --s) {
            EMSIM_TRY(launch_col(p->n1, COL_PROPAGATE, cb, nb, st));
            rb.slice = slices + (long long)s * npix;
            rb.phi = w.phi + (long long)(s - s0) * nwave;
            if (reduce) {
                rb.grad = w.part;
                rb.grad_img_stride = npix;
            } else {
                rb.grad = grad_slices + (long long)s * npix;
                rb.grad_img_stride = slices_stride;
            }
            EMSIM_TRY(launch_row(p->n2, s > 0 ? (ROW_IFFT | ROW_GRAD | ROW_TRANSMIT | ROW_FFT) : (ROW_IFFT | ROW_GRAD),
                                 rb, nb, st));
            if (reduce) {
                reduce_images_kernel<<<grid_for(npix), 256, 0, st>>>(w.part, grad_slices + (long long)s * npix, npix,
                                                                     nb);
                EMSIM_CHECK_LAUNCH();
            }
        }
    }
    return EMSIM_GB300_OK;
}

}  // extern "C"
