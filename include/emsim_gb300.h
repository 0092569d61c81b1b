/*
 * emsim_gb300 - C ABI of the GB300 (sm_103a) multislice engine for emsim.
 *
 * Plain pointers and sizes only.  Device pointers point to CUDA global memory on the
 * device that was current when the plan was created; "stream" is a cudaStream_t passed
 * as void* (NULL = legacy default stream).  Complex arrays are interleaved float32
 * (re, im) pairs, row-major, C-contiguous, exactly the cufftComplex layout the reference
 * extension uses.  Every entry point returns EMSIM_GB300_OK (0) or an error code; the
 * message of the last failure on the calling thread is returned by
 * emsim_gb300_last_error().  Work is enqueued asynchronously on "stream"; nothing here
 * synchronises the device except plan creation.  Plans and the library's per-device state
 * (twiddle table, error word, static buffers) belong to the device's primary context:
 * after cudaDeviceReset of a device, create new plans and make no call that relies on
 * state set up before the reset.
 *
 * Reference interfaces replaced (paths inside the emsim project):
 *   emsim::cuda::WavePropagator    emsim/backend/cuda_ext/src/WavePropagator.h:15-41,
 *                                  pybind wrapper wave_kernel_cuda.cpp:28-143
 *   emsim::cuda::OneSliceBuilder   emsim/backend/cuda_ext/src/SliceBuilder.h,
 *   emsim::cuda::MultiSlicesBuilder  pybind wrapper slice_kernel_cuda.cpp:80-214
 */
#ifndef EMSIM_GB300_H
#define EMSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMSIM_GB300_ABI_VERSION 1

enum {
    EMSIM_GB300_OK = 0,
    EMSIM_GB300_ERR_INVALID = 1,     /* bad argument (null pointer, size, shape) */
    EMSIM_GB300_ERR_CUDA = 2,        /* CUDA runtime error (message has details) */
    EMSIM_GB300_ERR_UNSUPPORTED = 3, /* valid request this build does not handle */
    EMSIM_GB300_ERR_DEVICE = 4       /* plan used on a device other than its own */
};

typedef struct emsim_gb300_wave_plan emsim_gb300_wave_plan;
typedef struct emsim_gb300_slice_plan emsim_gb300_slice_plan;

/* ABI version (EMSIM_GB300_ABI_VERSION). */
int emsim_gb300_abi_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char* emsim_gb300_last_error(void);

/* Synchronise the current device, then read and clear its device error word: 0 when
 * no kernel gave up; 1 when a pipelined kernel's bounded wait for a tile copy timed out
 * (its results are then invalid).  No reference counterpart: the reference reports
 * CUDA errors on stderr only (WavePropagator.cu:18-20). */
int emsim_gb300_check_device_error(int* code);

/* Read the current device's error word without synchronising the device and without
 * clearing it: kernels that have not finished are not reflected, so call it after the
 * host has waited (event, stream or device synchronisation) for the work it checks.
 * The word lives in mapped page-locked host memory.  No reference counterpart. */
int emsim_gb300_peek_device_error(int* code);

/* Limit (ns of GPU global time) of the bounded mbarrier waits of the TMA-pipelined and
 * tensor-core passes, process-wide; at least 1 ms, default 2 s.  After a timed-out wait a
 * kernel still waits at least the default for its own copy in flight before it exits.
 * No reference counterpart. */
int emsim_gb300_set_wait_limit_ns(unsigned long long ns);
unsigned long long emsim_gb300_get_wait_limit_ns(void);

/* Self-test of the timeout path: one CTA waits, bounded by limit_ns (1 us .. 2 s), on an
 * mbarrier that nothing arrives at, records the timeout in the device error word exactly
 * as a pipelined pass does, and writes 1 (the wait completed) or 0 (it gave up) to
 * *completed (device int).  Nothing is in flight, so the context stays usable.
 * No reference counterpart. */
int emsim_gb300_wait_timeout_probe(unsigned long long limit_ns, int* completed, void* stream);

/* ---------------------------------------------------------------------------------
 * Wave propagator.  Replaces WavePropagator(n1, n2, d1, d2, waveLength,
 * relativityGamma) (cuda_ext/src/WavePropagator.cu:14-21; python side
 * backend/wave_propagator_cuda.py:26-31).  wave_length in Angstrom, relativity_gamma
 * dimensionless (both FP64; sigma = gamma * lambda is formed in FP64).
 * All wave operations below take n_batch >= 1 images of shape (n1, n2) stored
 * back to back; input and output may alias (in-place).
 * ------------------------------------------------------------------------------- */
int emsim_gb300_wave_plan_create(int n1, int n2, double d1, double d2, double wave_length,
                                 double relativity_gamma, emsim_gb300_wave_plan** plan);
int emsim_gb300_wave_plan_destroy(emsim_gb300_wave_plan* plan);

/* psi = sqrt(dose * d1 * d2) everywhere (wave_propagator_base.py:25-29). */
int emsim_gb300_init_wave(emsim_gb300_wave_plan* plan, double electron_dose, void* wave_out,
                          int n_batch, void* stream);

/* psi * exp(i sigma V) (WavePropagator.cu:27-29, kernel WavePropagator_kernel.cu:12-43).
 * slice: (n1, n2) float32, shared by all images when slice_batch_stride == 0, else
 * slice_batch_stride floats apart. */
int emsim_gb300_slice_transmit(emsim_gb300_wave_plan* plan, const void* wave, const float* slice,
                               long long slice_batch_stride, void* wave_out, int n_batch, void* stream);

/* IFFT(P(dz) * bandlimit * FFT(psi)) / N (WavePropagator.cu:32-42,
 * kernel WavePropagator_kernel.cu:46-94). */
int emsim_gb300_space_propagate(emsim_gb300_wave_plan* plan, const void* wave, double dz, void* wave_out,
                                int n_batch, void* stream);

/* transmit then space-propagate (WavePropagator.cu:56-60). */
int emsim_gb300_singleslice_propagate(emsim_gb300_wave_plan* plan, const void* wave, const float* slice,
                                      long long slice_batch_stride, double dz, void* wave_out, int n_batch,
                                      void* stream);

/* the multislice loop over slices (n_slices, n1, n2) float32 (WavePropagator.cu:62-70).
 * slices_batch_stride: floats between the slice stacks of consecutive images (0 = shared). */
int emsim_gb300_multislice_propagate(emsim_gb300_wave_plan* plan, const void* wave, const float* slices,
                                     int n_slices, long long slices_batch_stride, double dz, void* wave_out,
                                     int n_batch, void* stream);

/* objective lens: IFFT(exp(-i chi) * aperture * FFT(psi)) / N
 * (WavePropagator.cu:44-54, kernel WavePropagator_kernel.cu:97-145). */
int emsim_gb300_lens_propagate(emsim_gb300_wave_plan* plan, const void* wave, double cs_mm, double defocus,
                               double aperture, void* wave_out, int n_batch, void* stream);

/* Partially coherent image (no counterpart in the reference, whose README lists the
 * partially coherent CTF as future work): for each exit wave b,
 *   image_out[b] = sum_k weights[k] * |IFFT(H_k * E_s * aperture * FFT(psi_b)) / N|^2
 * with H_k = exp(-i chi) at defocus[k] (focal spread as an incoherent sum over defocus
 * values, e.g. Gauss-Hermite nodes) and E_s = exp(-(pi a / lambda)^2 |grad chi / 2 pi|^2)
 * the quasi-coherent envelope of an illumination semi-angle a (rad; 0 = coherent).
 * work: lens_incoherent_workspace_size(plan, n_batch) bytes of device memory. */
size_t emsim_gb300_lens_incoherent_workspace_size(const emsim_gb300_wave_plan* plan, int n_batch);
int emsim_gb300_lens_intensity_incoherent(emsim_gb300_wave_plan* plan, const void* exit_wave, int n_batch,
                                          double cs_mm, const double* defocus, const double* weights,
                                          int n_defocus, double illumination_angle, double aperture,
                                          float* image_out, void* work, size_t work_bytes, void* stream);

/* |psi|^2 (pipe.py:81-82). n = number of complex elements. */
int emsim_gb300_intensity(const void* wave, float* intensity_out, long long n, void* stream);

/* Fused image formation for n_batch images (pipe.py:46-55, 79-84 after the slices exist):
 * init_wave(dose) -> multislice over (n_slices, n1, n2) -> lens -> |psi|^2.  The plane
 * wave is generated in registers and the exit wave is only written when
 * exit_wave_out != NULL.  defocus_host: n_defocus values in host memory; image b uses
 * defocus_host[b % n_defocus] and slice stack b * slices_batch_stride.
 * wave_work: device scratch of n_batch * n1 * n2 complex64 (contents undefined on
 * return); image_out: (n_batch, n1, n2) float32. */
int emsim_gb300_multislice_image(emsim_gb300_wave_plan* plan, const float* slices, int n_slices,
                                 long long slices_batch_stride, double dz, double electron_dose, double cs_mm,
                                 const double* defocus_host, int n_defocus, double aperture, float* image_out,
                                 void* wave_work, void* exit_wave_out, int n_batch, void* stream);

/* ---------------------------------------------------------------------------------
 * Slice builder.  Replaces OneSliceBuilder(scatFac, nElems, n1, n2, d1, d2) and
 * MultiSlicesBuilder(scatFac, nElems, nSlices, n1, n2, dz, d1, d2)
 * (cuda_ext/src/SliceBuilder.cu:12-32, 78-100).  scattering_factors_host:
 * (n_elems, n1, n2/2+1) float32 in HOST memory, the half-spectrum layout of
 * slice_builder_base.py:30-33; it is copied (the reference borrows a device buffer).
 * n_slices = 1 gives the one-slice builder.  symmetric_bandlimit != 0 applies the
 * circular band-limit of make_one_slice / make_multi_slices(symmetric_bandlimit=True)
 * (slice_builder_numpy.py:18-26, 37-44).
 * ------------------------------------------------------------------------------- */
int emsim_gb300_slice_plan_create(const float* scattering_factors_host, int n_elems, int n_slices, int n1,
                                  int n2, double dz, double d1, double d2, int symmetric_bandlimit,
                                  emsim_gb300_slice_plan** plan);
int emsim_gb300_slice_plan_destroy(emsim_gb300_slice_plan* plan);

/* Histogram of atoms per element (SliceBuilder_kernel.cu:9-61 one slice, 64-123 multi).
 * coords: (n_atoms, 3) float32 device, columns (z, x, y), rows grouped by element in
 * the order of elem_counts; elem_counts: (n_elems,) uint32 device.  out: float32
 * (n_elems, n1, n2) resp. (n_elems, n_slices, n1, n2); fully written (no pre-zeroing
 * needed).  Counts are exact integers and independent of execution order. */
int emsim_gb300_bin_atoms_one_slice(emsim_gb300_slice_plan* plan, const float* coords, unsigned n_atoms,
                                    const uint32_t* elem_counts, float* out, void* stream);
int emsim_gb300_bin_atoms_multi_slices(emsim_gb300_slice_plan* plan, const float* coords, unsigned n_atoms,
                                       const uint32_t* elem_counts, float* out, void* stream);

/* Bytes of device workspace emsim_gb300_make_slices needs for this plan. */
size_t emsim_gb300_make_slices_workspace_size(const emsim_gb300_slice_plan* plan);

/* Projected-potential slices from histograms (SliceBuilder.cu:39-64, 108-133 plus the
 * band-limit of slice_builder_cuda.py:88-99 and the clip at 1e-13).
 * hist: (n_elems, n_slices, n1, n2) float32 device; out: (n_slices, n1, n2) float32.
 * workspace: device buffer of at least emsim_gb300_make_slices_workspace_size bytes,
 * 256-byte aligned. */
int emsim_gb300_make_slices(emsim_gb300_slice_plan* plan, const float* hist, float* out, void* workspace,
                            size_t workspace_bytes, void* stream);

/* Bytes of device workspace emsim_gb300_build_slices needs for n_atoms atoms of
 * n_batch molecules. */
size_t emsim_gb300_build_slices_workspace_size(const emsim_gb300_slice_plan* plan, unsigned n_atoms, int n_batch);

/* Slices of n_batch molecules straight from their atoms: the composition
 * make_slices(bin_atoms_multi_slices(...)) of pot.build_multi_slices (pot.py:29-48,
 * slice_builder_cuda.py:63-70) without materialising the (n_elems, n_slices, n1, n2)
 * histogram.  Atoms are binned with the same rule, counting-sorted into
 * (molecule, element, slice pair, row) buckets, and the row transforms of the binned
 * atoms are summed exactly in 64-bit fixed point, so the result is deterministic.
 * coords: (n_atoms, 3) float32 device, molecules back to back, each grouped by element;
 * elem_counts: (n_batch, n_elems) uint32 device; out: (n_batch, n_slices, n1, n2) float32.
 * Needs n1, n2 powers of two in [8, 4096] (else EMSIM_GB300_ERR_UNSUPPORTED). */
int emsim_gb300_build_slices(emsim_gb300_slice_plan* plan, const float* coords, unsigned n_atoms,
                             const uint32_t* elem_counts, int n_batch, float* out, void* workspace,
                             size_t workspace_bytes, void* stream);

/* Voxel water (MultiSlicesBuilderBase.add_water, emsim/backend/slice_builder_base.py:134-147,
 * slice_builder_cuda.py:72-85): in every voxel of hist (n_elems, n_slices, n1, n2) float32
 * that is empty for all elements, add Poisson(w) oxygens to element o_index and
 * Poisson(2 w) hydrogens to element h_index, w = water_num_dens * d1 * d2 * dz.  The
 * reference draws from an unseeded global generator; here voxel v draws from
 * Philox4x32-10 with counter (v, stream_id) and key seed, so a seed reproduces the water
 * exactly.  Needs 0 <= w <= 64. */
int emsim_gb300_add_water(emsim_gb300_slice_plan* plan, float* hist, int h_index, int o_index,
                          double water_num_dens, uint64_t seed, uint32_t stream_id, void* stream);

/* Band-limit of a slice stack (band_limit_specimen, emsim/tem.py:102-108): every slice of
 * slices (n_slices, n1, n2) float32 is low-passed with the disc k1^2 + k2^2 <= 4 r^2 / 9
 * (r = min(n1, n2) // 2, k the fftfreq integers) and its real part written to out (may
 * equal slices).  The reference transforms axes (0, 1) of the stack, which matches its
 * own layout only for cubic stacks; here each slice is filtered on its lateral axes.
 * n1, n2 powers of two in [8, 4096]. */
size_t emsim_gb300_band_limit_workspace_size(int n_slices, int n1, int n2);
int emsim_gb300_band_limit_slices(const float* slices, int n_slices, int n1, int n2, float* out, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------------
 * Slices without a workspace.  No counterpart in the reference.
 * For callers that cannot allocate device memory when they need slices - a plugin inside
 * a host program that owns all device memory through its own pool, or a loop that must
 * not allocate after start-up (cudaMalloc/cudaFree can synchronise the device).  Same
 * result as emsim_gb300_make_slices, with the intermediate kept in one static device
 * buffer of EMSIM_GB300_NOALLOC_SCRATCH_BYTES instead of a workspace; no cudaMalloc,
 * cudaFree or allocating library call.  A plan needing more scratch
 * (emsim_gb300_make_slices_workspace_size) is rejected with EMSIM_GB300_ERR_UNSUPPORTED.
 * Every GPU that loads this part of the library may hold the buffer until the process
 * exits.  All calls on a device share it and it keeps the last call's contents (nothing
 * in it needs to start at zero); calls that overlap on the GPU race on it.  The first
 * call on a device looks up the buffer's address; make it before any stream capture.
 * Like every plan, that address is invalid after cudaDeviceReset of the device; do not
 * call this on a device after resetting it.
 * ------------------------------------------------------------------------------- */
#define EMSIM_GB300_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int emsim_gb300_make_slices_noalloc(emsim_gb300_slice_plan* plan, const float* hist, float* out, void* stream);

/* Centralisation of n_mol molecules on the device (atoms.centralize, emsim/atoms.py:142-159,
 * and AtomList.space, atoms.py:37-47): for each molecule, shift = -r_min - (r_max - r_min)/2
 * and the extent of the shifted coordinates, in float32 exactly as numpy evaluates them.
 * coords: (n_atoms, 3) float32 device; atom_offsets: (n_mol + 1) uint32 device, molecule m
 * owning atoms [off[m], off[m + 1]) (every molecule non-empty); shift_out, space_out:
 * (n_mol, 3) float32 device.  When present_out != NULL (then z: (n_atoms) int32 device),
 * present_out[4m + w] bit b is set when Z = 32w + b occurs in molecule m (Z < 128), the
 * element set sort_elements_and_count (atoms.py:53-86) would find. */
int emsim_gb300_centralize(const float* coords, const int32_t* z, const uint32_t* atom_offsets, int n_mol,
                           float* shift_out, float* space_out, uint32_t* present_out, void* stream);

/* emsim_gb300_build_slices for molecules given as they come (pot.build_multi_slices after
 * atoms.centralize, pipe.py:46-52): atoms in any order with their atomic numbers z
 * (n_atoms) int32; molecule m's coordinates are shifted by shift[m] (float32 add, e.g. the
 * output of emsim_gb300_centralize) before binning and go to output image mol_slot[m]
 * (-1: skip); elem_of_z: (128) int32 device table, element index of each Z in the plan's
 * element order or -1 (atoms of absent elements are dropped).  Workspace as for
 * emsim_gb300_build_slices_workspace_size(plan, n_atoms, n_batch). */
int emsim_gb300_build_slices_z(emsim_gb300_slice_plan* plan, const float* coords, const int32_t* z, unsigned n_atoms,
                               const uint32_t* atom_offsets, int n_mol, const float* shift, const int32_t* mol_slot,
                               const int32_t* elem_of_z, int n_batch, float* out, void* workspace,
                               size_t workspace_bytes, void* stream);

/* Image formation straight from atoms with the slices built chunk by chunk: Pipe.run
 * without water (pipe.py:46-55, 79-84; pot.build_multi_slices pot.py:29-48, the slice
 * builders SliceBuilder.cu:108-133 and the propagator WavePropagator.cu:14-70) for n_batch
 * molecules of one element set and slice count, with memory O(chunk) instead of the
 * (n_batch, n_slices, n1, n2) slice stack.  The atoms (as for emsim_gb300_build_slices_z)
 * are bucketed once; then for each chunk of chunk_pairs slice pairs the slice passes fill
 * a chunk buffer and the multislice steps (plane wave first, the wave plan's propagator
 * for the slice plan's dz) run through it; last the lens and |psi|^2 into image_out
 * (n_batch, n1, n2) float32.  Bitwise equal to emsim_gb300_build_slices_z followed by
 * emsim_gb300_multislice_image.  chunk_pairs < 1 or above the pair count: one chunk.
 * Both plans on the current device with equal sides, powers of two in [8, 4096]. */
size_t emsim_gb300_image_from_atoms_workspace_size(const emsim_gb300_slice_plan* plan, unsigned n_atoms,
                                                   int n_batch, int chunk_pairs);
int emsim_gb300_image_from_atoms_z(emsim_gb300_slice_plan* plan, emsim_gb300_wave_plan* wave_plan,
                                   const float* coords, const int32_t* z, unsigned n_atoms,
                                   const uint32_t* atom_offsets, int n_mol, const float* shift,
                                   const int32_t* mol_slot, const int32_t* elem_of_z, int n_batch,
                                   double electron_dose, double cs_mm, const double* defocus_host, int n_defocus,
                                   double aperture, float* image_out, int chunk_pairs, void* workspace,
                                   size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------------
 * Off-grid ("smooth") slices and their coordinate adjoint.  No counterpart in the
 * reference, whose potential is piecewise constant in the atom positions because atoms
 * are binned to pixel centres (SliceBuilder_kernel.cu:64-123).  The smooth build keeps
 * every step of emsim_gb300_build_slices (scattering factors, band-limit round trip,
 * clip at 1e-13, slice membership and box by the binning rule) but evaluates each atom's
 * structure factor exp(-2 pi i k . xi / n) at its exact lateral pixel coordinate
 * xi = (x - start) / d - 1/2 (Nyquist term cos(pi xi)); at bin centres it equals the
 * binned build.  Arguments as emsim_gb300_build_slices; slice sides powers of two in
 * [8, 4096].  Deterministic (fixed summation order).
 * ------------------------------------------------------------------------------- */
size_t emsim_gb300_smooth_workspace_size(const emsim_gb300_slice_plan* plan, unsigned n_atoms, int n_batch);

/* out: (n_batch, n_slices, n1, n2) float32 smooth slices. */
int emsim_gb300_build_slices_smooth(emsim_gb300_slice_plan* plan, const float* coords, unsigned n_atoms,
                                    const uint32_t* elem_counts, int n_batch, float* out, void* workspace,
                                    size_t workspace_bytes, void* stream);

/* dLoss/dcoords (n_atoms, 3) float32 for dLoss/dslices = grad_slices, given the slices the
 * smooth build returned for the same atoms.  Columns (z, x, y): z is 0 (slice membership
 * is piecewise constant), atoms outside the box get 0. */
int emsim_gb300_build_slices_smooth_adjoint(emsim_gb300_slice_plan* plan, const float* coords, unsigned n_atoms,
                                            const uint32_t* elem_counts, int n_batch, const float* slices,
                                            const float* grad_slices, float* grad_coords, void* workspace,
                                            size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------------
 * Differentiation of the fused image.  No counterpart in the reference (emsim has no
 * gradient); the forward is emsim_gb300_multislice_image (pipe.py:46-55, 79-84).
 * Loss gradient with respect to the slice potentials by the adjoint multislice:
 * dLoss/dV_s = 2 sigma Im(mu_s conj(phi_s)), phi_s the transmitted wave of slice s and
 * mu_s the back-propagated adjoint wave (conjugate Fresnel step, conjugate CTF).
 * Memory is O(sqrt(S)) waves: the forward stores the wave state every `every` slices,
 * the adjoint recomputes one segment of `every` slices at a time.  Wave sides must be
 * powers of two in [8, 4096] (else EMSIM_GB300_ERR_UNSUPPORTED).
 * ------------------------------------------------------------------------------- */

/* Number of checkpoint waves (each nb x n1 x n2 complex64) the checkpointed forward
 * stores: ceil(n_slices / every) - 1. */
int emsim_gb300_adjoint_checkpoints(int n_slices, int every);

/* Bytes of 256-byte-aligned device workspace emsim_gb300_multislice_image_adjoint needs:
 * (2 + min(every, n_slices)) waves of nb images, plus nb float images when the slices
 * are shared (slices_stride 0) by nb > 1 images. */
size_t emsim_gb300_adjoint_workspace_size(emsim_gb300_wave_plan* plan, int n_slices, int every, int nb,
                                          long long slices_stride);

/* emsim_gb300_multislice_image that also returns the complex image wave u (image = |u|^2)
 * in image_wave_out (nb x n1 x n2 complex64, also the work buffer) and stores the
 * checkpoints in ckpt (emsim_gb300_adjoint_checkpoints(n_slices, every) waves of nb
 * images; may be NULL when that is 0).  slices_stride: 0 (one stack shared by all nb
 * images) or the per-image stride in floats (>= n_slices * n1 * n2). */
int emsim_gb300_multislice_image_ckpt(emsim_gb300_wave_plan* plan, const float* slices, int n_slices,
                                      long long slices_stride, double dz, double dose, double cs_mm,
                                      const double* defocus_host, int n_defocus, double aperture, float* image_out,
                                      void* image_wave_out, void* ckpt, int every, int nb, void* stream);

/* Adjoint: grad_image (nb x n1 x n2 float32) = dLoss/dimage -> grad_slices = dLoss/dV.
 * Arguments as given to emsim_gb300_multislice_image_ckpt, with its image_wave and ckpt.
 * grad_slices has the layout of slices: per image at stride slices_stride, or, for
 * shared slices (stride 0), one (n_slices, n1, n2) stack holding the sum over the nb
 * images taken in image order (deterministic). */
int emsim_gb300_multislice_image_adjoint(emsim_gb300_wave_plan* plan, const float* slices, int n_slices,
                                         long long slices_stride, double dz, double dose, double cs_mm,
                                         const double* defocus_host, int n_defocus, double aperture,
                                         const float* grad_image, const void* image_wave, const void* ckpt,
                                         int every, float* grad_slices, void* workspace, size_t workspace_bytes,
                                         int nb, void* stream);

/* ---------------------------------------------------------------------------------
 * Pass tuning (no counterpart in the reference, whose FFTs are cuFFT / FFTW plans).
 * For wave passes of length n (power of two in [8, 4096]): whether the TMA-staged
 * persistent kernel may run (row_tma / col_tma: -1 or 1 = when it applies, 0 = never,
 * 2 = the kernels with 16 values per thread, lengths 256..4096) and the rows / columns per
 * tile (0 = built-in; a smaller power of two is honoured).  Tiles regroup independent rows
 * or columns only, so results are identical for every setting of one kernel family.
 * row_tma = -2 restores the built-in setting of length n (the other arguments are then
 * ignored): the 16-value kernels at 256 (4 rows, 8 columns per tile), 1024, 2048 (1 row
 * per tile) and 4096, the TMA kernels elsewhere, as measured fastest on GB300.  The table
 * is process-wide; emsim_gb300.autotune measures candidates and caches the choice per GPU
 * and size.
 * ------------------------------------------------------------------------------- */
int emsim_gb300_set_pass_tuning(int n, int row_tma, int row_rows, int col_tma, int col_cols);
/* out[0..3]: the current setting; out[4..7]: built-in tiles of the TMA row, simple row,
 * TMA column and simple column kernels for an n x n wave. */
int emsim_gb300_get_pass_tuning(int n, int* out);

/* ---------------------------------------------------------------------------------
 * Precision mode of the wave passes (no counterpart in the reference, which computes in
 * FP32 through cuFFT / FFTW).  0: plain FP32 Stockham passes (default).  1: split-BF16
 * tensor-core passes where they exist: 256-point rows and columns of the multislice step
 * (row inverse FFT + transmit + forward FFT, column FFT + propagate + inverse FFT) run as
 * two 16-point DFT GEMMs per transform on tcgen05 with bf16 hi + lo operands and fp32
 * accumulation (about 16 significant bits per stage); every other pass stays FP32.
 * Process-wide.
 * ------------------------------------------------------------------------------- */
int emsim_gb300_set_precision(int mode);
int emsim_gb300_get_precision(void);

/* ---------------------------------------------------------------------------------
 * Ragged batches: molecules of one lateral size with different slice counts in one call.
 * No counterpart in the reference, which builds and propagates one molecule at a time
 * (pipe.py:46-55, simulator.py:71-91).
 * ------------------------------------------------------------------------------- */

/* emsim_gb300_build_slices_z with a slice count per output image: slot_slices (n_batch)
 * int32 device, each in [1, plan n_slices].  Molecule m is binned along z with the
 * binning rule's axis for slot_slices[mol_slot[m]] slices (the axis pot.build_multi_slices
 * would use for that molecule alone) and its stack fills slices [0, slot_slices[slot]) of
 * its (n_slices, n1, n2) slot; the slices beyond are not computed and hold no defined
 * values. */
int emsim_gb300_build_slices_ragged(emsim_gb300_slice_plan* plan, const float* coords, const int32_t* z,
                                    unsigned n_atoms, const uint32_t* atom_offsets, int n_mol, const float* shift,
                                    const int32_t* mol_slot, const int32_t* elem_of_z, const int32_t* slot_slices,
                                    int n_batch, float* out, void* workspace, size_t workspace_bytes, void* stream);

/* emsim_gb300_multislice_image for nb images with their own slice counts
 * n_slices_host[i] >= 1, given in non-increasing order (sort the batch by slice count):
 * step s propagates only the images that still have a slice s, so no step is spent on
 * padding.  Image i reads its slice s at slices + i * slices_stride + s * n1 * n2
 * (slices_stride >= n_slices_host[0] * n1 * n2).  Wave sides powers of two in [8, 4096]. */
int emsim_gb300_multislice_image_ragged(emsim_gb300_wave_plan* plan, const float* slices, long long slices_stride,
                                        const int32_t* n_slices_host, double dz, double dose, double cs_mm,
                                        const double* defocus_host, int n_defocus, double aperture,
                                        float* image_out, void* wave_work, int nb, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EMSIM_GB300_H */
