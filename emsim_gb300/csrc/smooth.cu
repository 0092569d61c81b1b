// Off-grid ("smooth") projected-potential slices and their coordinate adjoint.
//
// emsim bins atoms to pixel centres before its Fourier-space build
// (SliceBuilder_kernel.cu:64-123, SliceBuilder.cu:108-133, band limit and clip of
// slice_builder_cuda.py:63-70, 88-99); its potential is piecewise constant in the atom
// positions.  The smooth build keeps every step but puts each atom at its exact lateral
// position: with the binning rule's start edge s0 and pixel d, xi = (x - s0)/d - 1/2
// (integer at a bin centre) and
//     S_e,s(k) = sum_a eps(k1, xi1_a) eps(k2, xi2_a),  eps(k, xi) = exp(-2 pi i k xi / n)
// with the Nyquist term (k = -n/2) symmetrised to cos(pi xi) so that the potential is
// real; V_s = max(IFFT(sum_e T_e S_e,s), 1e-13), T_e = F SF_e / N the plan's transfer.
// Slice membership and the drop of atoms outside the box use the binning rule, so the
// z derivative is zero; at bin centres the result equals the binned build.
//
// Phases: xi / n is reduced to a 32-bit fixed-point fraction U in FP64 once per atom;
// k * U mod 2^32 is exact in integer arithmetic, so each exponential needs one float
// sincospi of a value in [-1, 1).
//
// Forward: key atoms by (image, slice pair, element, slice parity), count, scan,
// scatter, rank-sort each bucket by atom index (deterministic summation order), then a
// register-tiled direct sum over the bucket's atoms for each 64 x 64 tile of the spectrum
// of a slice pair z = Z_2p + i Z_2p+1, an inverse 2-D FFT on the engine's passes, split
// and clip.  Adjoint: dL/dW = dL/dV where V was not clipped, FFT of the packed pair,
// B_e,s(k) = T_e(k) Gamma_s(k) with Gamma_s = conj(FFT(dL/dW_s)), and per atom
//     dL/dxi1 = Re sum_k B(k) deps(k1) eps(k2),  dL/dxi2 = Re sum_k B(k) eps(k1) deps(k2)
// as a tiled contraction over k2 then k1, partial sums per k1 tile reduced in order.
#include <cmath>
#include <cstdint>

#include "atoms_sort.h"
#include "binning.cuh"
#include "slice_plan.h"

using namespace emsim_gb300;

namespace {

constexpr int TILE = 64;
constexpr int THREADS = 256;
constexpr int SPEC_CHUNK = 32;  // atoms per shared-memory stage (spectrum)
constexpr int GRAD_CHUNK = 16;  // k2 per shared-memory stage (adjoint)
constexpr float CLIP = 1e-13f;

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct SmoothWs {
    size_t group_start, group_tmp, key, pha, count, start, scan_tmp, cursor, items, sorted, spec, part, total;
    long long n_keys;
    int n_pairs, k1_tiles;
};

SmoothWs smooth_ws(const emsim_gb300_slice_plan* p, unsigned n_atoms, int n_img) {
    SmoothWs w;
    const long long n_groups = (long long)n_img * p->n_elems;
    w.n_pairs = (p->n_slices + 1) / 2;
    w.n_keys = (long long)n_img * w.n_pairs * p->n_elems * 2;
    w.k1_tiles = (p->n1 + TILE - 1) / TILE;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    w.group_start = take(sizeof(unsigned) * (n_groups + 1));
    w.group_tmp = take(sizeof(unsigned) * scan_tmp_words(n_groups));
    w.key = take(sizeof(unsigned) * (size_t)n_atoms);
    w.pha = take(sizeof(uint2) * (size_t)n_atoms);
    w.count = take(sizeof(unsigned) * (size_t)w.n_keys);
    w.start = take(sizeof(unsigned) * ((size_t)w.n_keys + 1));
    w.scan_tmp = take(sizeof(unsigned) * scan_tmp_words(w.n_keys));
    w.cursor = take(sizeof(unsigned) * (size_t)w.n_keys);
    w.items = take(sizeof(unsigned) * (size_t)n_atoms);
    w.sorted = take(sizeof(unsigned) * (size_t)n_atoms);
    w.spec = take(sizeof(float2) * (size_t)n_img * w.n_pairs * p->n1 * p->n2);
    w.part = take(sizeof(float2) * (size_t)w.k1_tiles * n_atoms);
    w.total = o;
    return w;
}

int grid_for(long long n) {
    long long g = (n + THREADS - 1) / THREADS;
    return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

// xi / n reduced to [0, 1) as a 32-bit fixed-point fraction
__device__ __forceinline__ unsigned frac_u32(double xi, int n) {
    double t = xi / (double)n;
    t -= floor(t);
    return (unsigned)(unsigned long long)llrint(t * 4294967296.0);
}

__device__ __forceinline__ int signed_freq(int k, int n) { return k < (n + 1) / 2 ? k : k - n; }

// eps(k) and d eps / d xi for fixed-point fraction u of xi / n
__device__ __forceinline__ void eps_and_deriv(unsigned u, int k, int n, float2& e, float2& de) {
    const int ks = signed_freq(k, n);
    const unsigned ph = (unsigned)ks * u;  // k xi / n mod 1, exact
    const float t = (float)(int)ph * 4.656612873077393e-10f;  // 2^-31: angle pi t = 2 pi k xi / n
    float s, c;
    sincospif(t, &s, &c);
    if ((n & 1) == 0 && k == n / 2) {  // Nyquist: cos(pi xi); ks = -n/2, so s = sin(-pi xi)
        e = make_float2(c, 0.f);
        de = make_float2(3.14159265358979f * s, 0.f);  // d/dxi cos(pi xi) = -pi sin(pi xi)
    } else {
        e = make_float2(c, -s);
        const float w = -6.28318530717959f * (float)ks / (float)n;  // d/dxi = -2 pi i k / n
        de = make_float2(w * s, w * c);
    }
}

__device__ __forceinline__ float2 eps_only(unsigned u, int k, int n) {
    const int ks = signed_freq(k, n);
    const unsigned ph = (unsigned)ks * u;
    const float t = (float)(int)ph * 4.656612873077393e-10f;
    float s, c;
    sincospif(t, &s, &c);
    if ((n & 1) == 0 && k == n / 2) return make_float2(c, 0.f);
    return make_float2(c, -s);
}

// ---- keys, counting sort, deterministic order ---------------------------------------
struct KeyArgs {
    const float* coords;
    unsigned n_atoms;
    const unsigned* group_start;  // (n_groups + 1) prefix of per-(image, element) counts
    int n_groups, n_elems, n_pairs, n1, n2;
    BinAxis ax0, ax1, ax2;
    unsigned* key;
    uint2* pha;
    unsigned* count;
};

// key = ((image * n_pairs + slice / 2) * n_elems + element) * 2 + slice % 2
__global__ void smooth_key_kernel(KeyArgs a) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < (long long)a.n_atoms;
         r += (long long)gridDim.x * blockDim.x) {
        unsigned k = INVALID_BUCKET;
        uint2 ph = make_uint2(0u, 0u);
        if ((unsigned)r < a.group_start[a.n_groups]) {
            int lo = 0, hi = a.n_groups;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (a.group_start[mid + 1] > (unsigned)r) hi = mid;
                else lo = mid + 1;
            }
            const int img = lo / a.n_elems, e = lo - img * a.n_elems;
            const float z = a.coords[3 * r + 0], x = a.coords[3 * r + 1], y = a.coords[3 * r + 2];
            int s, i, j;
            if (bin_axis(z, a.ax0, s) && bin_axis(x, a.ax1, i) && bin_axis(y, a.ax2, j)) {
                k = (unsigned)((((long long)img * a.n_pairs + (s >> 1)) * a.n_elems + e) * 2 + (s & 1));
                ph.x = frac_u32(((double)x - (double)a.ax1.start) / (double)a.ax1.d - 0.5, a.n1);
                ph.y = frac_u32(((double)y - (double)a.ax2.start) / (double)a.ax2.d - 0.5, a.n2);
                atomicAdd(a.count + k, 1u);
            }
        }
        a.key[r] = k;
        a.pha[r] = ph;
    }
}

__global__ void smooth_scatter_kernel(const unsigned* key, unsigned n_atoms, unsigned* cursor, unsigned* items) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < (long long)n_atoms;
         r += (long long)gridDim.x * blockDim.x) {
        const unsigned k = key[r];
        if (k != INVALID_BUCKET) items[atomicAdd(cursor + k, 1u)] = (unsigned)r;
    }
}

// each bucket's atom indices in ascending order: rank = number of smaller indices
__global__ void __launch_bounds__(THREADS) bucket_rank_sort_kernel(const unsigned* start, const unsigned* items,
                                                                   unsigned* sorted, long long n_keys) {
    constexpr unsigned CH = 1024;
    __shared__ unsigned chunk[CH];
    for (long long b = blockIdx.x; b < n_keys; b += gridDim.x) {
        const unsigned s0 = start[b], m = start[b + 1] - s0;
        if (m == 0) continue;
        for (unsigned i0 = 0; i0 < m; i0 += blockDim.x) {
            const unsigned i = i0 + threadIdx.x;
            const unsigned v = i < m ? items[s0 + i] : 0u;
            unsigned rank = 0;
            for (unsigned c0 = 0; c0 < m; c0 += CH) {
                __syncthreads();
                for (unsigned t = threadIdx.x; t < CH && c0 + t < m; t += blockDim.x) chunk[t] = items[s0 + c0 + t];
                __syncthreads();
                const unsigned cm = m - c0 < CH ? m - c0 : CH;
                if (i < m)
                    for (unsigned t = 0; t < cm; ++t) rank += chunk[t] < v ? 1u : 0u;
            }
            if (i < m) sorted[s0 + rank] = v;
        }
        __syncthreads();
    }
}

// ---- forward: spectrum of each slice pair by direct summation ---------------------------
struct SpecArgs {
    const uint2* pha;
    const unsigned* start;
    const unsigned* sorted;
    const float* filt;  // (n_elems, n1, n2)
    float2* spec;       // (planes, n1, n2)
    int n1, n2, n_elems;
};

__global__ void __launch_bounds__(THREADS) smooth_spectrum_kernel(SpecArgs a) {
    __shared__ float2 e1s[SPEC_CHUNK][TILE];
    __shared__ float2 e2s[SPEC_CHUNK][TILE];
    __shared__ uint2 phs[SPEC_CHUNK];
    const int k2_0 = blockIdx.x * TILE, k1_0 = blockIdx.y * TILE;
    const long long plane = blockIdx.z;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float2 tot[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) tot[i][j] = make_float2(0.f, 0.f);
    for (int e = 0; e < a.n_elems; ++e) {
        float2 acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
        for (int q = 0; q < 2; ++q) {
            const long long key = (plane * a.n_elems + e) * 2 + q;
            const unsigned b0 = a.start[key], b1 = a.start[key + 1];
            for (unsigned c0 = b0; c0 < b1; c0 += SPEC_CHUNK) {
                const int cnt = b1 - c0 < (unsigned)SPEC_CHUNK ? (int)(b1 - c0) : SPEC_CHUNK;
                __syncthreads();
                if (threadIdx.x < SPEC_CHUNK)
                    phs[threadIdx.x] = threadIdx.x < cnt ? a.pha[a.sorted[c0 + threadIdx.x]] : make_uint2(0u, 0u);
                __syncthreads();
                for (int t = threadIdx.x; t < SPEC_CHUNK * TILE; t += THREADS) {
                    const int at = t / TILE, kk = t - at * TILE;
                    float2 v1 = make_float2(0.f, 0.f), v2 = make_float2(0.f, 0.f);
                    if (at < cnt) {
                        const int k1 = k1_0 + kk, k2 = k2_0 + kk;
                        if (k1 < a.n1) {
                            v1 = eps_only(phs[at].x, k1, a.n1);
                            if (q) v1 = make_float2(-v1.y, v1.x);  // odd slice of the pair: times i
                        }
                        if (k2 < a.n2) v2 = eps_only(phs[at].y, k2, a.n2);
                    }
                    e1s[at][kk] = v1;
                    e2s[at][kk] = v2;
                }
                __syncthreads();
                for (int at = 0; at < cnt; ++at) {
                    float2 x1[4], x2[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) x1[i] = e1s[at][ty + 16 * i];
#pragma unroll
                    for (int j = 0; j < 4; ++j) x2[j] = e2s[at][tx + 16 * j];
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            acc[i][j].x = fmaf(x1[i].x, x2[j].x, fmaf(-x1[i].y, x2[j].y, acc[i][j].x));
                            acc[i][j].y = fmaf(x1[i].x, x2[j].y, fmaf(x1[i].y, x2[j].x, acc[i][j].y));
                        }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k1 = k1_0 + ty + 16 * i, k2 = k2_0 + tx + 16 * j;
                if (k1 < a.n1 && k2 < a.n2) {
                    const float T = a.filt[((long long)e * a.n1 + k1) * a.n2 + k2];
                    tot[i][j].x = fmaf(T, acc[i][j].x, tot[i][j].x);
                    tot[i][j].y = fmaf(T, acc[i][j].y, tot[i][j].y);
                }
            }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k1 = k1_0 + ty + 16 * i, k2 = k2_0 + tx + 16 * j;
            if (k1 < a.n1 && k2 < a.n2) a.spec[(plane * a.n1 + k1) * a.n2 + k2] = tot[i][j];
        }
}

// pair (V_2p + i V_2p+1) -> slices, clipped
__global__ void split_clip_kernel(const float2* spec, float* out, int n_img, int n_pairs, int n_slices,
                                  long long npix) {
    const long long total = (long long)n_img * n_pairs * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long plane = i / npix, pix = i - plane * npix;
        const long long img = plane / n_pairs;
        const int p = (int)(plane - img * n_pairs);
        const float2 v = spec[i];
        float* o = out + (img * n_slices + 2 * p) * npix + pix;
        o[0] = fmaxf(v.x, CLIP);
        if (2 * p + 1 < n_slices) o[npix] = fmaxf(v.y, CLIP);
    }
}

// ---- adjoint -------------------------------------------------------------------------
// y = dL/dW_2p + i dL/dW_2p+1 with dL/dW = dL/dV where V was not clipped
__global__ void pack_grad_kernel(const float* slices, const float* grad, float2* y, int n_img, int n_pairs,
                                 int n_slices, long long npix) {
    const long long total = (long long)n_img * n_pairs * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long plane = i / npix, pix = i - plane * npix;
        const long long img = plane / n_pairs;
        const int p = (int)(plane - img * n_pairs);
        const long long o = (img * n_slices + 2 * p) * npix + pix;
        float re = slices[o] > CLIP ? grad[o] : 0.f, im = 0.f;
        if (2 * p + 1 < n_slices) im = slices[o + npix] > CLIP ? grad[o + npix] : 0.f;
        y[i] = make_float2(re, im);
    }
}

struct GradArgs {
    const uint2* pha;
    const unsigned* start;
    const unsigned* sorted;
    const float* filt;
    const float2* Y;  // (planes, n1, n2) FFT of the packed pair
    float2* part;     // (k1_tiles, n_atoms) partial (dL/dxi1, dL/dxi2) by sorted position
    unsigned n_atoms;
    long long n_keys;
    int n1, n2, n_elems;
};

__global__ void __launch_bounds__(THREADS) smooth_grad_kernel(GradArgs a) {
    __shared__ float2 bs[GRAD_CHUNK][TILE];   // B(k1, k2), k1 fastest
    __shared__ float2 e2s[GRAD_CHUNK][TILE];  // eps(k2) per atom, atom fastest
    __shared__ float2 d2s[GRAD_CHUNK][TILE];  // d eps(k2) / d xi2
    __shared__ uint2 phs[TILE];
    const int k1_0 = blockIdx.x * TILE;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const long long npix = (long long)a.n1 * a.n2;
    for (long long key = blockIdx.y; key < a.n_keys; key += gridDim.y) {
        const unsigned b0 = a.start[key], b1 = a.start[key + 1];
        if (b0 == b1) continue;
        const int q = (int)(key & 1);
        const long long rest = key >> 1;
        const int e = (int)(rest % a.n_elems);
        const long long plane = rest / a.n_elems;
        const float2* Yp = a.Y + plane * npix;
        const float* T = a.filt + (long long)e * npix;
        for (unsigned t0 = b0; t0 < b1; t0 += TILE) {
            const int cnt = b1 - t0 < (unsigned)TILE ? (int)(b1 - t0) : TILE;
            __syncthreads();
            if (threadIdx.x < TILE) phs[threadIdx.x] = threadIdx.x < cnt ? a.pha[a.sorted[t0 + threadIdx.x]] : make_uint2(0u, 0u);
            float2 R[4][4], Rd[4][4];  // [atom i][k1 j]
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) R[i][j] = Rd[i][j] = make_float2(0.f, 0.f);
            for (int c0 = 0; c0 < a.n2; c0 += GRAD_CHUNK) {
                __syncthreads();
                for (int t = threadIdx.x; t < GRAD_CHUNK * TILE; t += THREADS) {
                    const int kk = t / TILE, m = t - kk * TILE;
                    const int k2 = c0 + kk;
                    // B(k1, k2) = T_e(k) Gamma_s(k)
                    float2 b = make_float2(0.f, 0.f);
                    const int k1 = k1_0 + m;
                    if (k1 < a.n1 && k2 < a.n2) {
                        const float Tv = T[(long long)k1 * a.n2 + k2];
                        if (Tv != 0.f) {
                            const float2 yk = Yp[(long long)k1 * a.n2 + k2];
                            const float2 ym = Yp[(long long)((a.n1 - k1) % a.n1) * a.n2 + (a.n2 - k2) % a.n2];
                            // Gamma_2p = (conj(Y(k)) + Y(-k)) / 2, Gamma_2p+1 = i (conj(Y(k)) - Y(-k)) / 2
                            float2 g;
                            if (q == 0) g = make_float2(0.5f * (yk.x + ym.x), 0.5f * (ym.y - yk.y));
                            else g = make_float2(0.5f * (yk.y + ym.y), 0.5f * (yk.x - ym.x));
                            b = make_float2(Tv * g.x, Tv * g.y);
                        }
                    }
                    bs[kk][m] = b;
                    float2 ev = make_float2(0.f, 0.f), dv = make_float2(0.f, 0.f);
                    if (m < cnt && k2 < a.n2) eps_and_deriv(phs[m].y, k2, a.n2, ev, dv);
                    e2s[kk][m] = ev;
                    d2s[kk][m] = dv;
                }
                __syncthreads();
#pragma unroll 4
                for (int kk = 0; kk < GRAD_CHUNK; ++kk) {
                    float2 bb[4], ee[4], dd[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) bb[j] = bs[kk][tx + 16 * j];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        ee[i] = e2s[kk][ty + 16 * i];
                        dd[i] = d2s[kk][ty + 16 * i];
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            R[i][j].x = fmaf(bb[j].x, ee[i].x, fmaf(-bb[j].y, ee[i].y, R[i][j].x));
                            R[i][j].y = fmaf(bb[j].x, ee[i].y, fmaf(bb[j].y, ee[i].x, R[i][j].y));
                            Rd[i][j].x = fmaf(bb[j].x, dd[i].x, fmaf(-bb[j].y, dd[i].y, Rd[i][j].x));
                            Rd[i][j].y = fmaf(bb[j].x, dd[i].y, fmaf(bb[j].y, dd[i].x, Rd[i][j].y));
                        }
                }
            }
            // dL/dxi1 = Re sum_k1 deps1 R, dL/dxi2 = Re sum_k1 eps1 Rd over this k1 tile
            float g1[4], g2[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                g1[i] = 0.f;
                g2[i] = 0.f;
                const int at = ty + 16 * i;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k1 = k1_0 + tx + 16 * j;
                    if (at < cnt && k1 < a.n1) {
                        float2 ev, dv;
                        eps_and_deriv(phs[at].x, k1, a.n1, ev, dv);
                        g1[i] += dv.x * R[i][j].x - dv.y * R[i][j].y;
                        g2[i] += ev.x * Rd[i][j].x - ev.y * Rd[i][j].y;
                    }
                }
            }
            // reduce over the 16 lanes (tx) that share an atom, fixed order
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int off = 8; off >= 1; off >>= 1) {
                    g1[i] += __shfl_xor_sync(0xffffffffu, g1[i], off);
                    g2[i] += __shfl_xor_sync(0xffffffffu, g2[i], off);
                }
            if (tx == 0) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int at = ty + 16 * i;
                    if (at < cnt) a.part[(long long)blockIdx.x * a.n_atoms + t0 + at] = make_float2(g1[i], g2[i]);
                }
            }
        }
    }
}

// grad[atom] = (0, sum_tiles part.x / d1, sum_tiles part.y / d2), tiles in order
__global__ void grad_reduce_kernel(const float2* part, const unsigned* sorted, const unsigned* n_kept,
                                   unsigned n_atoms, int k1_tiles, float inv_d1, float inv_d2, float* grad) {
    const unsigned kept = *n_kept;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < (long long)kept;
         p += (long long)gridDim.x * blockDim.x) {
        float g1 = 0.f, g2 = 0.f;
        for (int t = 0; t < k1_tiles; ++t) {
            const float2 v = part[(long long)t * n_atoms + p];
            g1 += v.x;
            g2 += v.y;
        }
        const unsigned r = sorted[p];
        grad[3ull * r + 1] = g1 * inv_d1;
        grad[3ull * r + 2] = g2 * inv_d2;
    }
}

// shared front half: keys, counting sort, deterministic bucket order
int sort_atoms(const emsim_gb300_slice_plan* p, const SmoothWs& w, char* base, const float* coords, unsigned n_atoms,
               const uint32_t* elem_counts, int n_img, cudaStream_t st) {
    auto U = [&](size_t off) { return reinterpret_cast<unsigned*>(base + off); };
    const int n_groups = n_img * p->n_elems;
    EMSIM_TRY(scan_u32(elem_counts, U(w.group_start), n_groups, U(w.group_tmp), st));
    EMSIM_CHECK_CUDA(cudaMemsetAsync(U(w.count), 0, sizeof(unsigned) * (size_t)w.n_keys, st));
    if (n_atoms > 0) {
        KeyArgs k;
        k.coords = coords;
        k.n_atoms = n_atoms;
        k.group_start = U(w.group_start);
        k.n_groups = n_groups;
        k.n_elems = p->n_elems;
        k.n_pairs = w.n_pairs;
        k.n1 = p->n1;
        k.n2 = p->n2;
        k.ax0 = make_axis(p->n_slices, p->dz);
        k.ax1 = make_axis(p->n1, p->d1);
        k.ax2 = make_axis(p->n2, p->d2);
        k.key = U(w.key);
        k.pha = reinterpret_cast<uint2*>(base + w.pha);
        k.count = U(w.count);
        smooth_key_kernel<<<grid_for(n_atoms), THREADS, 0, st>>>(k);
        EMSIM_CHECK_LAUNCH();
    }
    EMSIM_TRY(scan_u32(U(w.count), U(w.start), w.n_keys, U(w.scan_tmp), st));
    EMSIM_CHECK_CUDA(cudaMemcpyAsync(U(w.cursor), U(w.start), sizeof(unsigned) * (size_t)w.n_keys,
                                     cudaMemcpyDeviceToDevice, st));
    if (n_atoms > 0) {
        smooth_scatter_kernel<<<grid_for(n_atoms), THREADS, 0, st>>>(U(w.key), n_atoms, U(w.cursor), U(w.items));
        EMSIM_CHECK_LAUNCH();
        const int blocks = (int)(w.n_keys < 152 * 16 ? w.n_keys : 152 * 16);
        bucket_rank_sort_kernel<<<blocks, THREADS, 0, st>>>(U(w.start), U(w.items), U(w.sorted), w.n_keys);
        EMSIM_CHECK_LAUNCH();
    }
    return EMSIM_GB300_OK;
}

int check_args(const emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms, const uint32_t* elem_counts,
               int n_img, void* ws, size_t ws_bytes, const SmoothWs& w) {
    EMSIM_TRY(check_slice_device(p));
    EMSIM_REQUIRE(p->fast, EMSIM_GB300_ERR_UNSUPPORTED,
                  "smooth slices: slice side is not a power of two in [8, 4096]");
    EMSIM_REQUIRE(n_img >= 1 && elem_counts && ws && (coords || n_atoms == 0), EMSIM_GB300_ERR_INVALID,
                  "smooth slices: bad arguments");
    EMSIM_REQUIRE(ws_bytes >= w.total, EMSIM_GB300_ERR_INVALID, "smooth slices: workspace too small");
    EMSIM_REQUIRE(((uintptr_t)ws & 255) == 0, EMSIM_GB300_ERR_INVALID, "smooth slices: workspace not 256-byte aligned");
    EMSIM_REQUIRE(w.n_keys < (long long)INVALID_BUCKET, EMSIM_GB300_ERR_UNSUPPORTED, "smooth slices: too many buckets");
    EMSIM_REQUIRE((long long)n_img * w.n_pairs <= 65535, EMSIM_GB300_ERR_UNSUPPORTED,
                  "smooth slices: more than 65535 image x slice-pair planes per call");
    return EMSIM_GB300_OK;
}

}  // namespace

extern "C" {

size_t emsim_gb300_smooth_workspace_size(const emsim_gb300_slice_plan* p, unsigned n_atoms, int n_batch) {
    if (!p || n_batch < 1) return 0;
    return smooth_ws(p, n_atoms, n_batch).total;
}

int emsim_gb300_build_slices_smooth(emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms,
                                    const uint32_t* elem_counts, int n_batch, float* out, void* workspace,
                                    size_t workspace_bytes, void* stream) {
    EMSIM_REQUIRE(p != nullptr, EMSIM_GB300_ERR_INVALID, "build_slices_smooth: null plan");
    const SmoothWs w = smooth_ws(p, n_atoms, n_batch < 1 ? 1 : n_batch);
    EMSIM_TRY(check_args(p, coords, n_atoms, elem_counts, n_batch, workspace, workspace_bytes, w));
    EMSIM_REQUIRE(out != nullptr, EMSIM_GB300_ERR_INVALID, "build_slices_smooth: null output");
    cudaStream_t st = (cudaStream_t)stream;
    char* base = (char*)workspace;
    EMSIM_TRY(sort_atoms(p, w, base, coords, n_atoms, elem_counts, n_batch, st));
    const int planes = n_batch * w.n_pairs;
    float2* spec = reinterpret_cast<float2*>(base + w.spec);
    SpecArgs s;
    s.pha = reinterpret_cast<const uint2*>(base + w.pha);
    s.start = reinterpret_cast<const unsigned*>(base + w.start);
    s.sorted = reinterpret_cast<const unsigned*>(base + w.sorted);
    s.filt = p->filt;
    s.spec = spec;
    s.n1 = p->n1;
    s.n2 = p->n2;
    s.n_elems = p->n_elems;
    const dim3 grid((p->n2 + TILE - 1) / TILE, (p->n1 + TILE - 1) / TILE, planes);
    smooth_spectrum_kernel<<<grid, THREADS, 0, st>>>(s);
    EMSIM_CHECK_LAUNCH();
    // unnormalised inverse 2-D FFT (T_e carries 1/N): columns, then rows
    ColArgs c;
    c.tw = p->tw;
    c.err = error_word();
    c.data = spec;
    c.img_stride = (long long)p->n1 * p->n2;
    c.n_rows = p->n1;
    c.n_cols = p->n2;
    EMSIM_TRY(launch_col(p->n1, COL_INV, c, planes, st));
    RowArgs r;
    r.tw = p->tw;
    r.err = error_word();
    r.in = spec;
    r.out = spec;
    r.in_img_stride = r.out_img_stride = (long long)p->n1 * p->n2;
    r.n_rows = p->n1;
    EMSIM_TRY(launch_row(p->n2, ROW_IFFT, r, planes, st));
    const long long npix = (long long)p->n1 * p->n2;
    split_clip_kernel<<<grid_for((long long)planes * npix), THREADS, 0, st>>>(spec, out, n_batch, w.n_pairs,
                                                                             p->n_slices, npix);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

int emsim_gb300_build_slices_smooth_adjoint(emsim_gb300_slice_plan* p, const float* coords, unsigned n_atoms,
                                            const uint32_t* elem_counts, int n_batch, const float* slices,
                                            const float* grad_slices, float* grad_coords, void* workspace,
                                            size_t workspace_bytes, void* stream) {
    EMSIM_REQUIRE(p != nullptr, EMSIM_GB300_ERR_INVALID, "build_slices_smooth_adjoint: null plan");
    const SmoothWs w = smooth_ws(p, n_atoms, n_batch < 1 ? 1 : n_batch);
    EMSIM_TRY(check_args(p, coords, n_atoms, elem_counts, n_batch, workspace, workspace_bytes, w));
    EMSIM_REQUIRE(slices && grad_slices && (grad_coords || n_atoms == 0), EMSIM_GB300_ERR_INVALID,
                  "build_slices_smooth_adjoint: null slices, gradient or output");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_atoms == 0) return EMSIM_GB300_OK;
    EMSIM_CHECK_CUDA(cudaMemsetAsync(grad_coords, 0, sizeof(float) * 3 * (size_t)n_atoms, st));
    char* base = (char*)workspace;
    EMSIM_TRY(sort_atoms(p, w, base, coords, n_atoms, elem_counts, n_batch, st));
    const int planes = n_batch * w.n_pairs;
    const long long npix = (long long)p->n1 * p->n2;
    float2* y = reinterpret_cast<float2*>(base + w.spec);
    pack_grad_kernel<<<grid_for((long long)planes * npix), THREADS, 0, st>>>(slices, grad_slices, y, n_batch,
                                                                            w.n_pairs, p->n_slices, npix);
    EMSIM_CHECK_LAUNCH();
    // unnormalised forward 2-D FFT: rows, then columns
    RowArgs r;
    r.tw = p->tw;
    r.err = error_word();
    r.in = y;
    r.out = y;
    r.in_img_stride = r.out_img_stride = npix;
    r.n_rows = p->n1;
    EMSIM_TRY(launch_row(p->n2, ROW_FFT, r, planes, st));
    ColArgs c;
    c.tw = p->tw;
    c.err = error_word();
    c.data = y;
    c.img_stride = npix;
    c.n_rows = p->n1;
    c.n_cols = p->n2;
    EMSIM_TRY(launch_col(p->n1, COL_FWD, c, planes, st));
    GradArgs g;
    g.pha = reinterpret_cast<const uint2*>(base + w.pha);
    g.start = reinterpret_cast<const unsigned*>(base + w.start);
    g.sorted = reinterpret_cast<const unsigned*>(base + w.sorted);
    g.filt = p->filt;
    g.Y = y;
    g.part = reinterpret_cast<float2*>(base + w.part);
    g.n_atoms = n_atoms;
    g.n_keys = w.n_keys;
    g.n1 = p->n1;
    g.n2 = p->n2;
    g.n_elems = p->n_elems;
    const dim3 grid(w.k1_tiles, (unsigned)(w.n_keys < 65535 ? w.n_keys : 65535));
    smooth_grad_kernel<<<grid, THREADS, 0, st>>>(g);
    EMSIM_CHECK_LAUNCH();
    const BinAxis a1 = make_axis(p->n1, p->d1), a2 = make_axis(p->n2, p->d2);
    grad_reduce_kernel<<<grid_for(n_atoms), THREADS, 0, st>>>(
        g.part, g.sorted, reinterpret_cast<const unsigned*>(base + w.start) + w.n_keys, n_atoms, w.k1_tiles,
        1.0f / a1.d, 1.0f / a2.d, grad_coords);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

}  // extern "C"
