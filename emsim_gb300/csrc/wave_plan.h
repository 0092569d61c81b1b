// The wave-propagator plan shared by the translation units that run multislice steps
// (wave_plan.cu: forward entry points; adjoint.cu: checkpointed forward and adjoint).
#pragma once

#include <mutex>

#include "engine.h"

namespace emsim_gb300 {

constexpr int PROP_SLOTS = 64;

}  // namespace emsim_gb300

struct emsim_gb300_wave_plan {
    int n1 = 0, n2 = 0;
    double d1 = 0, d2 = 0;
    double wave_length = 0, gamma = 0;
    float sigma = 0.f;           // gamma * lambda formed in FP64, rounded once
    float sigma_pi = 0.f;        // gamma * lambda / pi formed in FP64, rounded once
    float dfx = 0.f, dfy = 0.f;  // 1.0f / d / n in float32 (WavePropagator.cpp:19-20)
    double dfx64 = 0, dfy64 = 0;
    float filter2 = 0.f;  // (0.6667f * 0.5f / max(d1, d2))^2 in float32 (WavePropagator.cpp:21-23)
    bool fast = false;
    int device = 0;
    const float2* tw = nullptr;  // FFT twiddle table of the plan's device
    int* err = nullptr;          // device error word of the plan's device
    float2* tw1 = nullptr;       // generic path: exp(-2 pi i m / n1)
    float2* tw2 = nullptr;
    char* prop = nullptr;  // PROP_SLOTS x (float4 p1[n1] + float2 p2[n2]) propagator tables
    int* cut = nullptr;    // band-limit cutoff per row (bandlimit_cutoffs)
    int cut_max = -1;      // largest cutoff over the rows: columns beyond it are dead for propagation
    double prop_dz[emsim_gb300::PROP_SLOTS];
    // recorded on the stream that computed the slot's tables; callers on other streams
    // wait for it before reading them
    cudaEvent_t prop_ev[emsim_gb300::PROP_SLOTS] = {};
    int prop_used = 0;
    int prop_next = 0;
    std::mutex mu;
};

namespace emsim_gb300 {

// EMSIM_GB300_OK when p is a plan of the current device
int check_device(const emsim_gb300_wave_plan* p);
// device propagator tables for dz (computed on st the first time dz is seen)
int get_prop(emsim_gb300_wave_plan* p, double dz, cudaStream_t st, const float4** p1, const float2** p2);
// pass arguments with the plan's geometry filled in
ColArgs base_col(const emsim_gb300_wave_plan* p, float2* data);
RowArgs base_row(const emsim_gb300_wave_plan* p);
// lens constants: c1 (FP64), aperture^2 and the output scale
void set_lens(const emsim_gb300_wave_plan* p, ColArgs& a, double cs_mm, double aperture, float scale);

}  // namespace emsim_gb300
