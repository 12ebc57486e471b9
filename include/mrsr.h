/*
 * mrsr.h -- C ABI of the GB300 (sm_103a) subspace normal-operator library.
 *
 * Drop-in boundary for the GPU methods of MRISubspaceRecon.jl (published as
 * MRFingerprintingRecon.jl).  Each entry point replaces one reference method;
 * the reference file:line it replaces is given beside it.  A Julia package
 * extension binds these with `ccall` and keeps the reference's Julia
 * signatures.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers unless stated otherwise, in
 *    Julia's column-major layout with the reference's index order:
 *      images   x[r1, r2(, r3), k]            ComplexF32 (interleaved re,im)
 *      trj      trj[d, sample, frame]           Float32 in [-0.5, 0.5]
 *      data     data[sample, frame, coil(, rep)] ComplexF32
 *      U        U[frame, k(, rep)]              Float32 or ComplexF32
 *      cmaps    cmaps[r1, r2(, r3), coil]       ComplexF32 (the Julia shim
 *               stacks the reference's Vector{CuArray} once)
 *      sample_mask[sample, frame]               Bool (1 byte)
 *  - Every call takes an explicit CUDA stream (cudaStream_t, may be NULL for
 *    the legacy default stream) and is asynchronous unless noted.
 *  - Every function returns MRSR_OK (0) or an error code; the message is
 *    available from mrsr_last_error() (thread-local).  Device kernels never
 *    trap; kernels that can detect bad input write an error word that the
 *    host reads back and turns into MRSR_ERR_ARG.  The apply kernels that
 *    wait on mbarriers bound every wait; one that gives up writes the
 *    operator's error word and returns.  Applies are asynchronous, so the
 *    word is read where the library synchronises anyway (the end of
 *    mrsr_cg, mrsr_cg_stacked, mrsr_cg_noalloc, mrsr_cg_refined and
 *    mrsr_cg_batch_result)
 *    and by mrsr_normalop_check; a set word becomes MRSR_ERR_DEVICE and is
 *    cleared.
 *  - Handles are not thread-safe; different handles are independent.
 *  - There is no CPU fallback: without a usable sm_103a device every entry
 *    point returns MRSR_ERR_DEVICE or MRSR_ERR_CUDA.
 */
#ifndef MRSR_H
#define MRSR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  MRSR_OK = 0,
  MRSR_ERR_ARG = 1,         /* maps to ArgumentError / AssertionError */
  MRSR_ERR_CUDA = 2,
  MRSR_ERR_ALLOC = 3,
  MRSR_ERR_UNSUPPORTED = 4,
  MRSR_ERR_STATE = 5,
  MRSR_ERR_DEVICE = 6
};

/* Storage precision of the oversampled K-stack and the Toeplitz kernel. */
enum {
  MRSR_PREC_FP32 = 0, /* float32 everywhere (the reference's precision)   */
  MRSR_PREC_FP16 = 1, /* fp16 storage with per-tile scales, fp32 arithmetic */
  /* 2 is not used (rejected with MRSR_ERR_ARG) */
  MRSR_PREC_FP16_TC = 3     /* float32 stack and row passes; the Λ pass runs
                               its 64-point column DFTs on the tensor cores
                               (tcgen05, fp16 operands with per-tile
                               power-of-two scales, fp32 accumulation); NFFT
                               operators whose last grid length is 512     */
};

/* Density compensation of calculate_backprojection (src/BackProjection.jl:169-181). */
enum { MRSR_DCF_NONE = 0, MRSR_DCF_RADIAL_2D = 1, MRSR_DCF_RADIAL_3D = 2, MRSR_DCF_ARRAY = 3 };

/* Operator kinds reported by mrsr_normalop_info. */
enum { MRSR_KIND_NFFT = 0, MRSR_KIND_FFT = 1 };

typedef struct mrsr_normalop mrsr_normalop; /* opaque handle */
typedef void* mrsr_stream_t;                /* cudaStream_t   */

/* Message of the last error on this thread ("" if none). */
const char* mrsr_last_error(void);
/* Library ABI version (major*10000 + minor*100 + patch). */
int mrsr_version(void);

/* ---------------------------------------------------------------------
 * NFFTNormalOp(img_shape, trj, U; cmaps, sample_mask)
 *   replaces src/NFFTNormalOp.jl:29-42 and
 *   ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:1-13 (with the kernel
 *   precompute calculate_kernel_noncartesian, src:121-225 / ext:89-191, and
 *   calculate_kmask_indcs, src:106-118 / ext:75-86).
 * ndims 2 or 3; img_shape host array; trj (ndims, ns_per_frame, nt);
 * sample_mask may be NULL (all samples); U (nt, K) real (u_is_complex = 0:
 * real kernel, ext:140) or complex (ext:89); cmaps may be NULL (one unit coil,
 * the reference's default cmaps=(1,)).  2*img_shape must be 2,3,5-smooth.
 * Synchronous with respect to the host (it reads back sizes).
 */
int mrsr_nfft_normalop_create(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                              const float* trj, const uint8_t* sample_mask, const void* U,
                              int u_is_complex, int K, const float* cmaps, int ncoils, int precision,
                              mrsr_stream_t stream, mrsr_normalop** out);

/* NFFTNormalOp(img_shape, Λ, kmask_indcs; cmaps)
 *   replaces ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:22-70 (GPU packed Λ)
 *   and src/NFFTNormalOp.jl:51-86.
 * lambda_packed: (P, nk) column-major upper-triangle packing,
 * P = K(K+1)/2, index k1 + k2(k2-1)/2 (1-based k1 <= k2), real (Float32) or
 * complex; kmask_indcs: nk 1-based column-major indices into the
 * (2 img_shape) grid (Int64).  Checks the reference's @asserts (ext:28-30).
 */
int mrsr_nfft_normalop_from_lambda(int ndims, const int64_t* img_shape, int K, const void* lambda_packed,
                                   int lambda_is_complex, const int64_t* kmask_indcs, int64_t nk,
                                   const float* cmaps, int ncoils, int precision, mrsr_stream_t stream,
                                   mrsr_normalop** out);

/* FFTNormalOp(img_shape, trj::Integer, U; cmaps, sample_mask)
 *   replaces src/FFTNormalOp.jl:28-31 with calculate_kernel_cartesian (:81-97).
 * trj Int32 (ndims, ns_per_frame, nt) with grid coordinates (mod1 wrapping,
 * ifftshift applied as in :88); U (nt, K, nrep) real or complex.
 */
int mrsr_fft_normalop_create(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                             const int32_t* trj, const uint8_t* sample_mask, const void* U,
                             int u_is_complex, int K, int nrep, const float* cmaps, int ncoils,
                             int precision, mrsr_stream_t stream, mrsr_normalop** out);

/* FFTNormalOp(M, U; cmaps): replaces src/FFTNormalOp.jl:33-36 with :99-109.
 * M Bool (img_shape..., nt), U (nt, K) real or complex. */
int mrsr_fft_normalop_create_from_mask(int ndims, const int64_t* img_shape, int64_t nt, const uint8_t* M,
                                       const void* U, int u_is_complex, int K, const float* cmaps,
                                       int ncoils, int precision, mrsr_stream_t stream,
                                       mrsr_normalop** out);

/* FFTNormalOp(Λ; cmaps): replaces src/FFTNormalOp.jl:38-64.
 * lambda_full: ComplexF32 (K, K, img_shape...); kmask = Λ[1,1,:] .!= 0. */
int mrsr_fft_normalop_from_lambda(int ndims, const int64_t* img_shape, int K, const float* lambda_full,
                                  const float* cmaps, int ncoils, int precision, mrsr_stream_t stream,
                                  mrsr_normalop** out);

/* mul!(x, A, b, α, β):  y <- beta*y + alpha * A * x   (x, y: (img..., K))
 *   replaces ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218,
 *   src/NFFTNormalOp.jl:227-267 and src/FFTNormalOp.jl:111-149.
 * beta == 0 overwrites y (NaNs in y do not propagate, src:232-236).
 * x and y must not alias. */
int mrsr_normalop_apply(mrsr_normalop* op, const float* x, float* y, float alpha_re, float alpha_im,
                        float beta_re, float beta_im, mrsr_stream_t stream);

/* mul!(y, A, x, α, β) on host arrays: the reference's CPU method (src/NFFTNormalOp.jl:227-267,
 * src/FFTNormalOp.jl:111-149) for callers whose x and y live in host memory.  Replaces
 * copyto!(x_d, x); mul!(y_d, A, x_d, α, β); copyto!(y, y_d): x is copied into the operator's
 * own device buffer (made on first use; by the SMs over the CPU-GPU link when x is page-locked,
 * else by cudaMemcpyAsync); with one coil group, and y page-locked (addressable
 * by the device), the inverse row pass stores y straight into the host array over the
 * CPU-GPU link, so no copy back follows the apply; otherwise y returns by a copy.  Enqueued on
 * `stream`; y is final when `stream` has synchronised.  x and y must not alias. */
int mrsr_normalop_apply_host(mrsr_normalop* op, const float* x, float* y, float alpha_re, float alpha_im,
                             float beta_re, float beta_im, mrsr_stream_t stream);

/* Sizes of an operator (host array of 12 int64):
 * [kind, ndims, n1, n2, n3, K, ncoils, nk, lambda_is_complex, precision, P, launches_per_apply] */
int mrsr_normalop_info(const mrsr_normalop* op, int64_t* info);

/* Back the reference's A.prod!.A.kmask_indcs (1-based Int64, nk entries, device). */
int mrsr_normalop_get_kmask(const mrsr_normalop* op, int64_t* kmask_out, mrsr_stream_t stream);

/* Back the reference's A.prod!.A.Λ:
 *   NFFT op: packed (P, nk) Float32 (real kernel) or ComplexF32 (ext:104,156)
 *   FFT op:  ComplexF32 (K, K, nk) (src/FFTNormalOp.jl:331-332). */
int mrsr_normalop_get_lambda(const mrsr_normalop* op, void* out, mrsr_stream_t stream);

/* Per-pass device times of `iters` applies (milliseconds per apply, host
 * array of length launches_per_apply); used by the benchmark's roofline. */
int mrsr_normalop_profile(mrsr_normalop* op, const float* x, float* y, int iters, float* ms_per_pass,
                          mrsr_stream_t stream);

/* Synchronises `stream` and reports whether any apply enqueued on the operator
 * since the last check hit a bounded device wait that gave up (MRSR_ERR_DEVICE,
 * whose outputs are not valid); clears the word.  MRSR_OK otherwise.  The
 * reference has no counterpart: its operators run on the CPU. */
int mrsr_normalop_check(mrsr_normalop* op, mrsr_stream_t stream);

void mrsr_normalop_destroy(mrsr_normalop* op);

/* ---------------------------------------------------------------------
 * calculate_backprojection(data, trj, cmaps | img_shape; U, sample_mask,
 *                          density_compensation)
 *   replaces ext/MRISubspaceReconCUDAExt/BackProjection.jl:1-71 and
 *   src/BackProjection.jl:23-102 (float trajectories).
 * data (ns_per_frame, nt, ncoils); U (nt, K) real or complex, or NULL for
 * I(nt) (K = nt); cmaps (img..., ncoils) or NULL: out is then per coil,
 * (img..., K, ncoils) (src:23-60), else (img..., K).  dcf_kind MRSR_DCF_*;
 * dcf_array (masked-sample order, Float32) for MRSR_DCF_ARRAY.
 */
int mrsr_backprojection(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                        int ncoils, const float* data, const float* trj, const uint8_t* sample_mask,
                        const void* U, int u_is_complex, int K, const float* cmaps, int dcf_kind,
                        const float* dcf_array, float* out, mrsr_stream_t stream);

/* calculate_backprojection with an integer trajectory:
 *   replaces src/BackProjection.jl:104-156.  data (ns, nt, ncoils, nrep),
 *   U (nt, K, nrep). */
int mrsr_backprojection_cartesian(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                                  int ncoils, int nrep, const float* data, const int32_t* trj,
                                  const uint8_t* sample_mask, const void* U, int u_is_complex, int K,
                                  const float* cmaps, float* out, mrsr_stream_t stream);

/* ---------------------------------------------------------------------
 * Forward model (type-2 NUFFT with the reference tests' conventions,
 * test/reconstruct_radial.jl:62-74): data[s, t, c] =
 *   sum_r S_c(r) sum_k U[t,k] x_k(r) exp(-2 pi i k_{s,t}.(r - N/2)).
 * No counterpart in the reference package (its tests call NonuniformFFTs
 * directly); used to synthesise data on the device.
 */
int mrsr_forward_model(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt, int ncoils,
                       const float* x, const float* trj, const void* U, int u_is_complex, int K,
                       const float* cmaps, float* data_out, mrsr_stream_t stream);

/* ---------------------------------------------------------------------
 * GROG (src/GROG.jl).
 * grog_calib(data, trj, Nr): replaces src/GROG.jl:14-51.
 *   data (ns_per_frame, nt, ncoils, nrep) with ns_per_frame a multiple of Nr;
 *   lnG_out: ComplexF32 (ndims, Nc, Nc) -- lnG[d] = lnG_out[d, :, :].
 * grog_gridding!(data, trj, lnG, Nr, img_shape): replaces src/GROG.jl:73-102.
 *   data updated in place; trj_cart_out Int32 (ndims, ns_per_frame, nt),
 *   bit-exact with the reference's rounding.
 */
int mrsr_grog_calib(int ndims, int64_t nr, int64_t ns_per_frame, int64_t nt, int ncoils, int nrep,
                    const float* data, const float* trj, float* lnG_out, mrsr_stream_t stream);
int mrsr_grog_gridding(int ndims, const int64_t* img_shape, int64_t nr, int64_t ns_per_frame, int64_t nt,
                       int ncoils, int nrep, float* data, const float* trj, const float* lnG,
                       int32_t* trj_cart_out, mrsr_stream_t stream);

/* ---------------------------------------------------------------------
 * ESPIRiT coil sensitivities: espirit(kbp, img_shape, kernel_size;
 * eigThresh_1, eigThresh_2, nmaps) of MRICoilSensitivities.jl as
 * calculate_coil_maps calls it (src/CoilMaps.jl:55-57, :89-91); the reference's
 * GPU extension copies kbp to the host for it (ext/MRISubspaceReconCUDAExt/
 * CoilMaps.jl:29-31), this runs on the device.
 * kbp: centred calibration k-space (calib_shape..., ncoils) ComplexF32, DC at
 * calib / 2; maps_out (img_shape..., ncoils, nmaps) ComplexF32; eig_out
 * (img_shape..., nmaps) Float32 or NULL.  Signal subspace: singular vectors of
 * the calibration matrix with sigma >= eig_thresh_1 * sigma_max; maps: leading
 * eigenvectors of the image-space ESPIRiT operator, zero where the eigenvalue is
 * below eig_thresh_2, coil 1 real and non-negative.  2D, 1..32 coils,
 * nmaps 1..2 (else MRSR_ERR_UNSUPPORTED).  Synchronises the stream once per
 * Jacobi sweep of the calibration SVD; asynchronous after that. */
int mrsr_espirit(int ndims, const int64_t* img_shape, const int64_t* calib_shape, int ncoils, const float* kbp,
                 const int64_t* kernel_size, double eig_thresh_1, double eig_thresh_2, int nmaps, float* maps_out,
                 float* eig_out, mrsr_stream_t stream);

/* ---------------------------------------------------------------------
 * cg(A, b; maxiter, reltol, abstol) with x0 = 0 as IterativeSolvers.jl 0.9
 * runs it on the LinearOperator (call sites test/*.jl, src/CoilMaps.jl:136).
 * Vectors ComplexF32; each thread sums its few elements' products in float32,
 * the rest of every inner product and norm, and alpha/beta, in float64 on the
 * device (deterministic).  Stops after maxiter iterations or once
 * ||r|| <= max(reltol*||b||, abstol).  iters_out / resnorm_out are host
 * pointers (may be NULL); the call synchronises the stream to return them.
 * The iterations run as launches of CUDA graphs (8 and 1 iterations) that the
 * first solve on an operator records into its workspace.
 */
int mrsr_cg(mrsr_normalop* op, const float* b, float* x, int maxiter, double reltol, double abstol,
            int* iters_out, double* resnorm_out, mrsr_stream_t stream);

/* CG as mrsr_cg, without any device allocation (no counterpart in the
 * reference).  For callers that cannot let the library call cudaMalloc: a host
 * framework that hands out all device memory through its own pool, or a loop
 * that must not allocate after start-up.  The three work vectors live in a
 * static 32 MiB device array compiled into the library, so the solve is
 * limited to about 1.39 million unknowns (nimg * K); larger operators are
 * rejected with MRSR_ERR_UNSUPPORTED.  The first call on each device looks up
 * the array's device address (cudaGetSymbolAddress).  Every call synchronises
 * `stream` at its end (it reads the iteration count and residual back) and,
 * when a tolerance is set, every 8 iterations, so it cannot be called inside
 * a stream capture.  All calls share the one array: calls that overlap on the
 * GPU (other streams, other host threads) race and must be serialised by the
 * caller.  The operator itself must already exist. */
int mrsr_cg_noalloc(mrsr_normalop* op, const float* b, float* x, int maxiter, double reltol, double abstol,
                    int* iters_out, double* resnorm_out, mrsr_stream_t stream);

/* Stacked right-hand sides (reconstruct_coilwise, src/CoilMaps.jl:118-162:
 * `for i in 1:Nc; x[.., i] = cg(AᴴA, b[.., i]; maxiter)`, and its GPU form
 * ext/MRISubspaceReconCUDAExt/CoilMaps.jl:57-77).
 * mrsr_normalop_stack: from a float32 rank-1 operator src (K = 1), an operator
 * on nrhs (1..64) stacked images x (img..., nrhs) that applies src to every
 * plane independently (same kernel, kmask and coil maps; planes are not mixed).
 * mrsr_cg_stacked runs one independent cg per plane of such an operator in
 * one set of launches: each plane has its own alpha, beta, tolerance test and
 * iteration count, exactly as nrhs separate mrsr_cg calls would (the planes'
 * reductions are the same arithmetic, so results agree to float32 rounding).
 * iters_out / resnorm_out receive nrhs entries (host, may be NULL). */
int mrsr_normalop_stack(const mrsr_normalop* src, int nrhs, mrsr_stream_t stream, mrsr_normalop** out);
int mrsr_cg_stacked(mrsr_normalop* op, const float* b, float* x, int maxiter, double reltol, double abstol,
                    int* iters_out, double* resnorm_out, mrsr_stream_t stream);

/* Mixed-precision iterative refinement (no counterpart in the reference):
 * outer residual r = b - A_hi x with the float32 operator, inner CG on a
 * reduced-precision operator op_lo (fp16 or fp16-tc), until
 * ||r|| <= tol*||b||, max_outer, or an outer step that more than doubles
 * the residual (that step is undone and relres_out is the residual before
 * it).  op_lo and op_hi must describe the same operator. */
int mrsr_cg_refined(mrsr_normalop* op_lo, mrsr_normalop* op_hi, const float* b, float* x, int inner_iters,
                    int max_outer, double tol, int* outer_out, double* relres_out, mrsr_stream_t stream);

/* Relaxed mixed-precision CG (no counterpart in the reference): cg(A, b;
 * maxiter, reltol, abstol) as mrsr_cg runs it (x0 = 0, IterativeSolvers'
 * recurrence), whose operator products use the float32 op_hi while
 * ||r|| > switch_relres * ||b|| and the reduced-precision op_lo (fp16 or
 * fp16-tc) after that, on the same recurrence (no restart).  Product errors
 * taken at a large residual move a CG iterate the most, so the first few
 * iterations stay float32 and the rest run on the faster operator; the iterate
 * stays close to the float32 / float64 CG iterate of the same iteration count
 * (switch_relres = 0.05 on 20 iterations: ~5e-4 from float64).  0 runs every
 * product on op_hi, >= 1 every product on op_lo.  iters_out, hi_iters_out (the
 * float32 iterations) and resnorm_out are host pointers (may be NULL); the
 * call synchronises the stream, once per float32 iteration.  op_lo and op_hi
 * must describe the same operator; the vectors live in op_hi's workspace. */
int mrsr_cg_relaxed(mrsr_normalop* op_lo, mrsr_normalop* op_hi, const float* b, float* x, int maxiter,
                    double reltol, double abstol, double switch_relres, int* iters_out, int* hi_iters_out,
                    double* resnorm_out, mrsr_stream_t stream);

/* ---------------------------------------------------------------------
 * Serving support (no counterpart in the reference).
 *
 * mrsr_normalop_share: a new operator on src's Toeplitz kernel and kmask,
 * which it shares by reference count (not copied), with its own coil maps
 * (cmaps (img..., ncoils) or NULL) and work stacks.  precision may differ
 * from src's (the fp16 copy of the kernel is made once and shared too).
 * Destroying src first is allowed.
 */
int mrsr_normalop_share(const mrsr_normalop* src, const float* cmaps, int ncoils, int precision,
                        mrsr_stream_t stream, mrsr_normalop** out);

/* A batch of independent fixed-iteration solves recorded once into one CUDA
 * graph, one graph branch per entry, so that the entries overlap on the
 * device and a launch costs one cudaGraphLaunch.
 *   ops_hi == NULL or ops_hi[i] == NULL: entry i is cg(A, b; maxiter =
 *     inner_iters, reltol = 0) with x0 = 0 on ops_lo[i] (the kernels of
 *     mrsr_cg, without its tolerance test).
 *   ops_hi[i] != NULL: mixed-precision refinement with a fixed schedule,
 *     x = 0, r = b; outer_steps times { d = cg(ops_lo[i], r; inner_iters);
 *     x += d; r = b - ops_hi[i] x } (ops_hi[i] float32, ops_lo[i] fp16).
 * Pointers b[i], x[i] are baked into the graph: each launch solves again with
 * the current contents of b[i]; x[i] is overwritten.  No operator may appear
 * in two entries.  Relaunching before the previous launch finished is
 * ordered only by the stream the caller passes.
 * mrsr_cg_batch_result (synchronises): plain entries give the iterations run
 * and the final ||r||; refined entries give outer_steps and ||r|| / ||b||. */
typedef struct mrsr_cg_batch mrsr_cg_batch; /* opaque handle */
int mrsr_cg_batch_create(mrsr_normalop* const* ops_lo, mrsr_normalop* const* ops_hi, const float* const* b,
                         float* const* x, int n, int inner_iters, int outer_steps, mrsr_stream_t stream,
                         mrsr_cg_batch** out);
/* A batch of relaxed mixed-precision solves: the fixed-schedule form of
 * mrsr_cg_relaxed for graph capture.  Entry i is cg(A, b; maxiter = iters,
 * reltol = 0) from x0 = 0 on one recurrence (vectors in ops_hi[i]'s workspace)
 * whose first hi_iters products use ops_hi[i] (float32) and the others
 * ops_lo[i] (a reduced-precision share of the same kernel and maps).
 * hi_iters = iters gives the float32 solve, 0 the reduced one.  Launch,
 * result (iterations and final ||r||) and destroy as for the batches above. */
int mrsr_cg_batch_create_relaxed(mrsr_normalop* const* ops_lo, mrsr_normalop* const* ops_hi, const float* const* b,
                                 float* const* x, int n, int iters, int hi_iters, mrsr_stream_t stream,
                                 mrsr_cg_batch** out);
int mrsr_cg_batch_launch(mrsr_cg_batch* batch, mrsr_stream_t stream);
int mrsr_cg_batch_result(mrsr_cg_batch* batch, int i, int* iters_out, double* resnorm_out);
void mrsr_cg_batch_destroy(mrsr_cg_batch* batch);

#ifdef __cplusplus
}
#endif

#endif /* MRSR_H */
