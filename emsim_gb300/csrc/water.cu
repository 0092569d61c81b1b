// Voxel water on the device (MultiSlicesBuilderBase.add_water, emsim/backend/
// slice_builder_base.py:134-147 and slice_builder_cuda.py:72-85): in every voxel that is
// empty for all elements, add Poisson(w) oxygens and Poisson(2 w) hydrogens,
// w = water_num_dens * d1 * d2 * dz (physics.py:6).
//
// The reference draws from numpy's / cupy's unseeded global generator; here the draws are
// counter-based and seeded, so a seed reproduces the water exactly on any launch shape:
// voxel v uses Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC11) with counter (v_lo, v_hi, stream, 0) and key (seed_lo, seed_hi);
// word 0 drives the oxygen draw, word 1 the hydrogen draw.  Poisson variates come from
// sequential inversion in FP64 (u = word * 2^-32, F_k = sum_{j<=k} e^-l l^j / j!), bounded
// at MAX_COUNT.
#include <cmath>
#include <cstdint>

#include "slice_plan.h"

using namespace emsim_gb300;

namespace {

constexpr int MAX_COUNT = 255;

__host__ __device__ inline void philox_round(uint32_t (&c)[4], const uint32_t (&k)[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c[0] = hi1 ^ c[1] ^ k[0];
    c[1] = lo1;
    c[2] = hi0 ^ c[3] ^ k[1];
    c[3] = lo0;
}

__host__ __device__ inline void philox4x32_10(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
    uint32_t k[2] = {k0, k1};
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
        philox_round(c, k);
    }
}

// smallest k with u < F_k (F_k the Poisson(l) distribution function, e_l = exp(-l))
__device__ __forceinline__ int poisson_inv(uint32_t word, double l, double e_l) {
    const double u = (double)word * 2.3283064365386963e-10;  // 2^-32
    double p = e_l, F = e_l;
    int k = 0;
    while (u >= F && k < MAX_COUNT) {
        ++k;
        p = p * l / (double)k;
        F += p;
    }
    return k;
}

struct WaterArgs {
    float* hist;       // (n_elems, n_vox) float32
    long long n_vox;   // n_slices * n1 * n2
    int n_elems, h_index, o_index;
    double l_o, e_o, l_h, e_h;
    uint32_t seed_lo, seed_hi, stream;
};

__global__ void add_water_kernel(WaterArgs a) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < a.n_vox;
         v += (long long)gridDim.x * blockDim.x) {
        bool vacant = true;
        for (int e = 0; e < a.n_elems; ++e) vacant = vacant && a.hist[(long long)e * a.n_vox + v] == 0.f;
        if (!vacant) continue;
        uint32_t c[4] = {(uint32_t)v, (uint32_t)((unsigned long long)v >> 32), a.stream, 0u};
        philox4x32_10(c, a.seed_lo, a.seed_hi);
        const int o = poisson_inv(c[0], a.l_o, a.e_o);
        const int h = poisson_inv(c[1], a.l_h, a.e_h);
        if (o) a.hist[(long long)a.o_index * a.n_vox + v] += (float)o;
        if (h) a.hist[(long long)a.h_index * a.n_vox + v] += (float)h;
    }
}

}  // namespace

extern "C" int emsim_gb300_add_water(emsim_gb300_slice_plan* p, float* hist, int h_index, int o_index,
                                     double water_num_dens, uint64_t seed, uint32_t stream_id, void* stream) {
    EMSIM_TRY(check_slice_device(p));
    EMSIM_REQUIRE(hist != nullptr, EMSIM_GB300_ERR_INVALID, "add_water: null histogram");
    EMSIM_REQUIRE(h_index >= 0 && h_index < p->n_elems && o_index >= 0 && o_index < p->n_elems && h_index != o_index,
                  EMSIM_GB300_ERR_INVALID, "add_water: hydrogen and oxygen must be two of the plan's elements");
    const double w = water_num_dens * p->d1 * p->d2 * p->dz;
    EMSIM_REQUIRE(w >= 0.0 && w <= 64.0, EMSIM_GB300_ERR_UNSUPPORTED,
                  "add_water: mean waters per voxel must lie in [0, 64]");
    WaterArgs a;
    a.hist = hist;
    a.n_vox = (long long)p->n_slices * p->n1 * p->n2;
    a.n_elems = p->n_elems;
    a.h_index = h_index;
    a.o_index = o_index;
    a.l_o = w;
    a.e_o = std::exp(-w);
    a.l_h = 2.0 * w;
    a.e_h = std::exp(-2.0 * w);
    a.seed_lo = (uint32_t)seed;
    a.seed_hi = (uint32_t)(seed >> 32);
    a.stream = stream_id;
    long long blocks = (a.n_vox + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    add_water_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}
