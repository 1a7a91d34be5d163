/*
 * fluxoptics_gb300.h -- C ABI of the GB300-native scalar-propagation hot path of
 * FluxOptics.jl (angular-spectrum and Rayleigh-Sommerfeld propagation, Phase and
 * Mask modulation, the AS_BPM split-step march, their adjoints and gradients, the
 * SquaredIntensityDifference metric, and the Fista / ClampProx / TVProx update).
 *
 * Conventions
 *   - Every entry point returns FO_OK (0) or an FO_ERR_* code; fo_last_error()
 *     returns the message of the last failure on the calling thread.
 *   - Arrays are borrowed device pointers owned by the caller.  A batch of fields
 *     is `batch` contiguous complex-float (re, im) planes of ny rows x nx columns,
 *     x fastest: exactly the memory of a Julia CuArray{ComplexF32}(nx, ny, dims...)
 *     with the trailing dims flattened into `batch`.
 *   - `direction` is FO_FORWARD (+1) or FO_BACKWARD (-1), the reference's
 *     sign(Forward) / sign(Backward) (src/optical_components/OpticalComponents.jl:97-98).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     stream-ordered and do not synchronise; none allocates device memory except
 *     the *_create functions, so sequences of calls can be captured in a CUDA
 *     graph (fo_graph_*).
 *   - Plans (fo_prop_plan, fo_chain, fo_bpm, fo_sid, fo_tv) own their device
 *     workspace and are destroyed with the matching *_destroy.
 *   - Grid sizes of the propagators are powers of two from 16 to 4096 along
 *     each axis (RSProp: the padded size, >= 2n-1, must be one).
 */
#ifndef FLUXOPTICS_GB300_H
#define FLUXOPTICS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FO_API __attribute__((visibility("default")))
#else
#define FO_API
#endif

#define FO_OK 0
#define FO_ERR_ARG 1         /* null pointer / bad value */
#define FO_ERR_SHAPE 2       /* unsupported or mismatched sizes */
#define FO_ERR_ALLOC 3       /* device allocation failed */
#define FO_ERR_CUDA 4        /* a CUDA call failed */
#define FO_ERR_TIMEOUT 5     /* a bounded device wait gave up */
#define FO_ERR_UNSUPPORTED 6 /* feature not available in this build */

#define FO_FORWARD 1
#define FO_BACKWARD (-1)

/* Plan flags */
#define FO_FLAG_AUTOTUNE 1 /* time every launch shape of the passes and keep the fastest */
#define FO_FOURIER_TRAINABLE 2 /* fo_fourier_create: allocate the spectra of fo_fourier_gradient */
#define FO_FLAG_GRAD_SPECTRA 2 /* fo_asprop_create(_ex): allocate the spectra of fo_prop_z_gradient */
#define FO_FLAG_DEVICE_Z 4     /* fo_asprop_create_ex: keep what fo_prop_set_z needs to rebuild a filtered plan */

/* Modulation kinds (fo_mod.kind) */
#define FO_MOD_NONE 0
#define FO_MOD_PHASE 1 /* u *= cis(s*phi)        param: float[ny*nx]        */
#define FO_MOD_MASK 2  /* u *= m (conj(m) if s<0) param: complex float[ny*nx] */
#define FO_MOD_DN 3    /* u *= cis(s*scale/lambda_b*dn)  param: float[ny*nx]   */
#define FO_MOD_TEA 4   /* u *= r_b*cis(s*k_b*h) (conj(r_b) if s<0)  param: float[ny*nx] height,
                          field_coef: float[batch][4] = {k_b = 2 pi dn(lambda_b)/lambda_b, Re r_b, Im r_b, 0} */

/* ---------------------------------------------------------------------- */
/* Library                                                                 */
/* ---------------------------------------------------------------------- */

/* Version as major*10000 + minor*100 + patch. */
FO_API int fo_version(void);

/* Message of the last failed call on this thread ("" if none). */
FO_API const char* fo_last_error(void);

/* Blocks until all work on `stream` is done; reports device-side errors. */
FO_API int fo_stream_synchronize(void* stream);

/* Synchronises `stream`, then reads and clears the device error word of the
 * current device: FO_ERR_TIMEOUT when a kernel's bounded wait (an mbarrier wait
 * on a TMA copy or a grid barrier of the ragged launch, limit FO_WAIT_NS
 * nanoseconds, default 1 s) gave up since the last call.  Such a kernel returns without finishing its tile; the context stays
 * usable.  No counterpart in the reference (it has no device-side waits). */
FO_API int fo_device_status(void* stream);

/* Per-pass timing of the calls made between begin and end (eager calls only,
 * not graph replays): CUDA events around every pass launch.  ms[3] / launches[3]
 * receive the summed device time and the launch count of the single row
 * transforms, the fused inverse+forward row passes and the column passes.
 * No counterpart in the reference (it has no profiling hooks). */
FO_API int fo_profile_begin(void);
FO_API int fo_profile_end(double* ms, int* launches);

/* ---------------------------------------------------------------------- */
/* Free-space propagators                                                  */
/* ---------------------------------------------------------------------- */

typedef struct fo_prop_plan_s* fo_prop_plan;

/*
 * ASProp: u <- IFFT2(H . FFT2(u)) with the on-axis angular-spectrum transfer
 * function H = cis(2 pi z sqrt(n0^2/lambda^2 - fx^2 - fy^2)) (complex sqrt, so
 * evanescent waves decay), conj(H(-z)) for z < 0, conj(H) for the Backward
 * direction.  H is evaluated in FP64 and stored as complex float, once per
 * distinct wavelength.  `lambdas` holds one wavelength per field (n_lambdas ==
 * batch) or one shared wavelength (n_lambdas == 1).
 * Replaces: ASProp(u, ds, z; n0) -- src/optical_components/freespace_propagators/
 * angular_spectrum.jl:1-12 (as_kernel), :78-146 (ASKernelProp), :193-234 (ASProp),
 * with FourierWrapper (fourier/fourier_wrapper.jl:1-5) and compute_ft!/compute_ift!
 * (src/FFTutils.jl:13-28; CUFFT plans in src/cuda/CUDAExt.jl:29-35).
 */
FO_API int fo_asprop_create(fo_prop_plan* plan, int nx, int ny, int batch, double dx, double dy,
                            const double* lambdas, int n_lambdas, double z, double n0, int flags);

/*
 * Options of fo_asprop_create_ex; a zeroed struct gives fo_asprop_create.
 *   paraxial    : Fresnel transfer function
 *                 cis(-pi lm z ((fx+f0x)^2 + (fy+f0y)^2) - off + 2 pi z / lm),
 *                 off = track_tilts ? 2 (f0x fx + f0y fy) : 0, lm = lambda / n0
 *   tilts       : (theta_x, theta_y) in radians, one pair shared or one per field; any
 *                 non-zero tilt selects the tilted kernel
 *                 cis(2 pi z (sqrt(1/lm^2 - (fx+f0x)^2 - (fy+f0y)^2) + off)),
 *                 off = track_tilts ? (f0x fx + f0y fy) lm : 0, f0 = sin(theta) / lm
 *                 (conj(H(-z)) for z < 0)
 *   filter      : optional host callback filling re/im with the filter's value at n
 *                 frequencies (fx, fy) -- shifted by f0 for the tilted kernel, as the
 *                 reference evaluates filter(fx + f0x, fy + f0y) -- called once per
 *                 table at plan creation.
 * One transfer function is built per distinct (wavelength, tilts).
 * Replaces: as_paraxial_kernel / tilted_as_kernel / the filter argument of
 * ASKernelProp (angular_spectrum.jl:27-76, :78-146) and ParaxialProp.
 */
typedef void (*fo_filter_fn)(const double* fx, const double* fy, long long n, double* re, double* im,
                             void* ctx);
typedef struct {
  int paraxial;
  int track_tilts;
  const double* tilts; /* NULL or 2 * n_tilts angles */
  int n_tilts;         /* 1 or batch */
  fo_filter_fn filter; /* NULL: no filter */
  void* filter_ctx;
} fo_as_options;

FO_API int fo_asprop_create_ex(fo_prop_plan* plan, int nx, int ny, int batch, double dx, double dy,
                               const double* lambdas, int n_lambdas, double z, double n0,
                               const fo_as_options* options, int flags);

/*
 * In-place 2-D DFT of every field on the plan's grid (an ASProp or Fourier plan; a
 * padded RSProp plan is rejected).  FFTW's fft / ifft conventions, which the
 * reference's compute_ft! / compute_ift! use, and their adjoints:
 *   FO_FFT_FORWARD          F u     = sum_x u(x) e^{-2 pi i k.x / n} (unnormalised)
 *   FO_FFT_INVERSE          F^H u / (nx ny)
 *   FO_FFT_FORWARD_ADJOINT  F^H u   (the adjoint of FO_FFT_FORWARD)
 *   FO_FFT_INVERSE_ADJOINT  F u / (nx ny)  (the adjoint of FO_FFT_INVERSE)
 * Replaces: FourierOperator(u, direct) -- fourier/fourier_operator.jl:37-83 with
 * FFTutils.jl:13-28; the adjoints are the pull-backs of its two transforms.
 */
#define FO_FFT_FORWARD 0
#define FO_FFT_INVERSE 1
#define FO_FFT_FORWARD_ADJOINT 2
#define FO_FFT_INVERSE_ADJOINT 3
FO_API int fo_fft2(fo_prop_plan plan, void* u, int mode, void* stream);

/*
 * RSProp: zero-pad to (px, py) = the smallest powers of two >= (2nx-1, 2ny-1),
 * FFT, multiply by H_RS = FFT of the Rayleigh-Sommerfeld impulse response
 * h = dx dy/(2 pi) cis(k r)/r (z/r)(1/r - i k) sampled on the circular offset
 * grid, inverse FFT, crop the top-left nx x ny block.  The circular convolution
 * on >= 2n-1 points equals the reference's linear convolution on the cropped
 * block.  Padding is never materialised.
 * Replaces: RSProp(u, ds, z) -- src/optical_components/freespace_propagators/
 * rayleigh_sommerfeld.jl:1-12 (rs_kernel), :38-91 (RSKernelProp), :128-169 (RSProp),
 * convolution_kernel.jl:1-55 and utilities/pad_crop_operators.jl:291-356.
 */
FO_API int fo_rsprop_create(fo_prop_plan* plan, int nx, int ny, int batch, double dx, double dy,
                            const double* lambdas, int n_lambdas, double z, int flags);

/*
 * Padding and cropping of `batch` fields.  fo_pad writes px x py fields whose values
 * are pad_re + i pad_im except the nx x ny block whose first element is at column ox,
 * row oy, which holds the src field; fo_crop writes the nx x ny block at (ox, oy) of
 * each px x py src field.  The offsets are 0-based (the reference's `offset`).  src and
 * dst must not overlap.
 * Replaces: pad! / crop! (src/optical_components/utilities/pad_crop_operators.jl:1-16,
 * :61-79) as PadOperator / CropOperator and PadCropOperator (:122-356) apply them.
 */
FO_API int fo_pad(const void* src, int nx, int ny, void* dst, int px, int py, int batch, int ox, int oy,
                  double pad_re, double pad_im, void* stream);
FO_API int fo_crop(const void* src, int px, int py, void* dst, int nx, int ny, int batch, int ox, int oy,
                   void* stream);

/*
 * Fourier-domain modulators (FourierPhase / FourierMask): u <- IFFT2(w . FFT2(u)) with
 * w = cis(phi) (kind FO_MOD_PHASE) or m (FO_MOD_MASK), the parameter given on the
 * FFT-ordered frequency grid (fftfreq, function_to_array(f, ns, ds, true)); conj(w)
 * for the Backward direction.  The plan is a propagator: fo_propagate and chains run
 * it through the fused passes, so a Fourier filter between propagators costs no extra
 * pass.  fo_fourier_set rebuilds w from the parameter on the stream (call it after the
 * parameter changes; graph-capturable).  fo_fourier_gradient (plans created with
 * FO_FOURIER_TRAINABLE) computes the parameter gradient from the modulator's input
 * u_saved and the adjoint dv at its output, both in real space:
 *   phase: dphi = s sum_b Im(cis(-s phi) A_b conj(U_b)),  mask: dm = sum_b conj_s(A_b conj(U_b)),
 * U = FFT2(u_saved), A = FFT2(dv) (unnormalised), s = direction.
 * Replaces: FourierPhase / FourierMask = FourierWrapper(ft, Phase|Mask, ift)
 * (fourier/fourier_phase.jl:29-65, fourier/fourier_mask.jl, fourier/fourier_wrapper.jl:1-5,
 * fourier/fourier_operator.jl:37-83).
 */
/*
 * ASPropZ (trainable distance) on an ASProp plan of any kernel (on axis, tilted or
 * paraxial, with or without a filter): fo_prop_set_z rebuilds the transfer functions
 * in FP64 from the distance held in device memory (float z, read on the stream, so an
 * iteration that updates z can be captured as one graph).  A filtered plan must be
 * created with FO_FLAG_DEVICE_Z or FO_FLAG_GRAD_SPECTRA, which keep its filter values.
 * fo_prop_z_gradient (plan created with FO_FLAG_GRAD_SPECTRA) writes to *dz the
 * derivative of the loss with respect to z, from the propagator's input u_saved and
 * the adjoint du at its output: Re sum_b sum_k U conj(G) dH/dz / N with U = FFT2(u_saved),
 * G = FFT2(du), dH/dz = i R H, conjugated for the Backward direction, where R is the
 * kernel's phase rate: 2 pi (kz + off) for the on-axis and tilted kernels (kz =
 * sqrt(complex(1/lm^2 - (f+f0)^2)), conj for z < 0, off the tilt-tracking term) and
 * -pi lm (f+f0)^2 + 2 pi / lm for the paraxial one -- what Zygote computes through the
 * reference's propagate(u, ::ASPropZ) (angular_spectrum.jl:274-344).
 */
FO_API int fo_prop_set_z(fo_prop_plan plan, const float* z, void* stream);
FO_API int fo_prop_z_gradient(fo_prop_plan plan, const float* z, const void* u_saved, const void* du,
                              int direction, float* dz, void* stream);

FO_API int fo_fourier_create(fo_prop_plan* plan, int nx, int ny, int batch, int flags);
FO_API int fo_fourier_set(fo_prop_plan plan, int kind, const void* param, void* stream);
FO_API int fo_fourier_gradient(fo_prop_plan plan, int kind, const void* param, const void* u_saved,
                               const void* dv, void* grad, int direction, void* stream);

FO_API int fo_prop_destroy(fo_prop_plan plan);

/* Padded transform sizes and the workspace the plan owns. */
FO_API int fo_prop_info(fo_prop_plan plan, int* fft_nx, int* fft_ny, size_t* workspace_bytes);

/*
 * Launch shapes the plan runs (chosen by the autotuner or the defaults): the row
 * and column pass variant indices and a readable name of each kernel, written
 * NUL-terminated into row_kernel / col_kernel (up to len bytes each; either may
 * be NULL).  No reference counterpart: FFT plans are opaque in FluxOptics.jl.
 */
FO_API int fo_prop_variants(fo_prop_plan plan, int* row_variant, int* col_variant, char* row_kernel,
                            char* col_kernel, int len);

/*
 * In-place propagation of u (batch x ny x nx complex float).  FO_BACKWARD applies
 * the exact adjoint (conj(H)).
 * Replaces: propagate!(u, p::ASProp|RSProp, dir) and backpropagate!
 * (src/optical_components/freespace_propagators/freespace.jl:29-63,
 * system/optical_sequence.jl:54-66).
 */
FO_API int fo_propagate(fo_prop_plan plan, void* u, int direction, void* stream);

/* ---------------------------------------------------------------------- */
/* Modulators (any nx, ny)                                                 */
/* ---------------------------------------------------------------------- */

/*
 * u *= cis(s*phi), phi (ny x nx float) broadcast over the batch; when u_saved is
 * not NULL the input is copied there first.
 * Replaces: propagate!/propagate_and_save!(u, p::Phase, dir) --
 * src/optical_components/modulators/phasemask.jl:90-113.
 */
FO_API int fo_phase_forward(void* u, const float* phi, void* u_saved, int nx, int ny, int batch,
                            int direction, void* stream);

/*
 * dv <- cis(-s*phi) dv and, when dphi is not NULL,
 * dphi = s * sum_batch Im(dv_new * conj(u_saved)).
 * Replaces: backpropagate_with_gradient!(dv, u_saved, dp, p::Phase, dir) --
 * phasemask.jl:96-98, :115-150, and compute_phase_gradient! for CuArray
 * (src/cuda/optical_components.jl:1-44).
 */
FO_API int fo_phase_backward(void* dv, const float* phi, const void* u_saved, float* dphi, int nx,
                             int ny, int batch, int direction, void* stream);

/* u *= m (conj(m) for FO_BACKWARD); saves the input when u_saved is not NULL.
 * Replaces: propagate!(u, p::Mask, dir; u_saved) -- modulators/mask.jl:241-261. */
FO_API int fo_mask_forward(void* u, const void* m, void* u_saved, int nx, int ny, int batch,
                           int direction, void* stream);

/* dm = sum_batch conj_dir(dv * conj(u_saved)) (when dm is not NULL), then
 * dv <- conj_dir(m, reverse(dir)) dv.
 * Replaces: backpropagate_with_gradient!(dv, u_saved, dp, p::Mask, dir) -- mask.jl:263-291. */
FO_API int fo_mask_backward(void* dv, const void* m, const void* u_saved, void* dm, int nx, int ny,
                            int batch, int direction, void* stream);

/*
 * TeaDOE (thin-element DOE, also TeaReflector with dn = 2): u *= r_b cis(s k_b h) on
 * every field b, with k_b = 2 pi dn(lambda_b) / lambda_b and r_b = r(lambda_b) given
 * per field in `field_coef` (device float[batch][4] = {k_b, Re r_b, Im r_b, 0});
 * the conjugate amplitude for s < 0.  The backward call applies the adjoint and,
 * when dh is not NULL, writes dh = sum_b s k_b Im(du_b conj(u_saved_b)).
 * Replaces: propagate!/propagate_and_save!/backpropagate_with_gradient! of TeaDOE
 * (modulators/tea_doe.jl:150-215).
 */
FO_API int fo_tea_forward(void* u, const float* h, const void* field_coef, void* u_saved, int nx, int ny,
                          int batch, int direction, void* stream);
FO_API int fo_tea_backward(void* dv, const float* h, const void* field_coef, const void* u_saved, float* dh,
                           int nx, int ny, int batch, int direction, void* stream);

/* ---------------------------------------------------------------------- */
/* Fused chains: mod_0 -> prop_0 -> mod_1 -> ... -> prop_{K-1} -> mod_K     */
/* ---------------------------------------------------------------------- */

typedef struct {
  int kind;          /* FO_MOD_* */
  const void* param; /* phi / dn: float[ny*nx]; mask: complex float[ny*nx] */
  void* saved;       /* forward: the modulation input is written here when not NULL
                        (batch x ny x nx complex float); backward: the saved input */
  void* grad;        /* backward: gradient written here when not NULL
                        (phase / dn: float[ny*nx]; mask: complex float[ny*nx]) */
  double scale;      /* FO_MOD_DN: kdz = 2 pi dz / cos(theta); unused otherwise */
  const void* field_coef; /* FO_MOD_TEA: device float[batch][4] per-field coefficients; else unused */
} fo_mod;

typedef struct fo_chain_s* fo_chain;

/*
 * A chain of K propagators on one grid (all ASProp, or all RSProp with equal
 * padding) and one batch, executed as 2K+1 fused passes: the inverse row
 * transform of each propagator, the modulation after it and the forward row
 * transform of the next propagator run in one pass.  The plans stay owned by the
 * caller and must outlive the chain.
 * Replaces: OpticalSystem / AbstractSequence propagation over a run of
 * propagators and modulators (system/optical_sequence.jl:54-66,
 * system/optical_system.jl:189-214, system/merge_rules.jl:45-52).
 */
FO_API int fo_chain_create(fo_chain* chain, int n_props, const fo_prop_plan* props);
FO_API int fo_chain_destroy(fo_chain chain);

/*
 * Field probes of the chain's forward calls: pre[k] receives the field entering
 * modulation slot k (after propagator k-1; pre[0] is the chain input) and post[k]
 * the field leaving it (before propagator k; post[n_props] is the chain output),
 * k = 0..n_props.  Each non-NULL pointer is a caller-owned batch x ny x nx complex
 * float array written by the row pass that applies slot k, so probes cost no extra
 * pass.  The pointers stay set for every later fo_chain_forward[_from|_sid] until
 * replaced; NULL arrays (or all-NULL entries) remove them.  Probes are not written
 * by the adjoint sweep.
 * Replaces: FieldProbe (system/field_probe.jl:31-43) collected into
 * result.probes by OpticalSystem (system/optical_system.jl:194-214).
 */
FO_API int fo_chain_set_probes(fo_chain chain, void* const* pre, void* const* post);

/* Forward through the chain, in place on u; mods has n_props+1 entries. */
FO_API int fo_chain_forward(fo_chain chain, void* u, const fo_mod* mods, int direction,
                            void* stream);

/* As fo_chain_forward, but the input is read from u_in (left unchanged) and the
 * result written to u: the source copy of the reference's system call
 * (sources/scalar_source.jl:69-72) fused into the first pass. */
FO_API int fo_chain_forward_from(fo_chain chain, const void* u_in, void* u, const fo_mod* mods,
                                 int direction, void* stream);

/*
 * Adjoint sweep in reverse order, in place on du.  For every mod with a grad
 * pointer the gradient is written (mods[k].saved must then hold the input saved
 * by the forward sweep).  When `sid` is not NULL the sweep is seeded with the
 * SquaredIntensityDifference pullback du = 4 dc_t (I_t - target_t) u_out computed
 * by that metric's last fo_sid_forward call on `u_out`; du's content is then
 * ignored.
 * Replaces: the rrule pullbacks of propagate!/Trainable components
 * (src/ChainRulesCoreExt.jl:21-111) chained through the system in reverse.
 */
typedef struct fo_sid_s* fo_sid;
FO_API int fo_chain_backward(fo_chain chain, void* du, const fo_mod* mods, int direction,
                             fo_sid sid, const void* u_out, void* stream);

/*
 * Forward through the chain (from u_in when not NULL, else in place on u) with
 * SquaredIntensityDifference evaluated on the result inside the last pass: the
 * same outputs as fo_chain_forward[_from] followed by fo_sid_forward(sid, u,
 * target, loss), without a separate read of u.  The residuals are kept in `sid`
 * for a seeded fo_chain_backward_ex.  When the metric's target slices have
 * different field counts the metric runs as its own pass instead.
 * Replaces: the forward half of Zygote.withgradient(metric, system) for
 * SquaredIntensityDifference -- system/optical_system.jl:189-214 followed by
 * compute_metric, src/metrics/squared_intensity_difference.jl:78-83.
 */
FO_API int fo_chain_forward_sid(fo_chain chain, const void* u_in, void* u, const fo_mod* mods,
                                int direction, fo_sid sid, const float* target, float* loss,
                                void* stream);

/* fo_chain_backward with flags.  FO_BWD_DISCARD_INPUT_GRAD: only the parameter
 * gradients are wanted (the chain's input is not trainable); the final write of
 * the input gradient is skipped and du is left holding scratch values. */
#define FO_BWD_DISCARD_INPUT_GRAD 1
FO_API int fo_chain_backward_ex(fo_chain chain, void* du, const fo_mod* mods, int direction,
                                fo_sid sid, const void* u_out, int flags, void* stream);

/*
 * Zygote.withgradient(metric, system) for a chain and SquaredIntensityDifference in
 * one call: the forward sweep from u_in (left unchanged) with the metric (loss[T]
 * receives the per-slice values), then the seeded adjoint sweep on du, which ends
 * holding the gradient with respect to u_in unless flags has
 * FO_BWD_DISCARD_INPUT_GRAD.  mods_fwd and mods_bwd describe the n_props + 1
 * modulation slots for the two sweeps (what fo_chain_forward_sid and
 * fo_chain_backward_ex would be given); trainable slots write their gradients.
 * u_out (nullable, not du) receives the output field.  u_in must not alias u_out or du
 * (the adjoint sweep reads it).  When the last slot is empty,
 * every target slice holds the same number of fields and no probes are set, the
 * forward sweep's last row pass and the adjoint sweep's first row pass run as one
 * pass, so the iteration reads and writes the fields once less: 4K + 1 passes
 * instead of 4K + 2.  Otherwise the result is that of the two separate calls.  The
 * values are the same bit for bit either way.
 * Replaces: Zygote.withgradient over the reference's rrules (src/ChainRulesCoreExt.jl:21-111)
 * for a system ending in a propagator with SquaredIntensityDifference
 * (src/metrics/squared_intensity_difference.jl:58-90) as the loss.
 */
FO_API int fo_chain_withgradient_sid(fo_chain chain, const void* u_in, void* u_out, void* du,
                                     const fo_mod* mods_fwd, const fo_mod* mods_bwd, int direction, fo_sid sid,
                                     const float* target, float* loss, int flags, void* stream);

/* ---------------------------------------------------------------------- */
/* AS_BPM                                                                  */
/* ---------------------------------------------------------------------- */

typedef struct fo_bpm_s* fo_bpm;

/*
 * Split-step march through n_slices slices of thickness/n_slices: half step,
 * (n_slices-1) x [dn phase, full step], dn phase, half step, with the dn phase
 * cis(s*kdz/lambda*dn_k), kdz = 2 pi dz / cos_correction.  The adjoint needs the
 * slice inputs: every `checkpoint_every`-th one is kept by fo_bpm_forward(save=1)
 * and the others are recomputed segment by segment (checkpoint_every = 1 keeps
 * all, like the reference; 0 picks round(sqrt(n_slices))).
 * Replaces: AS_BPM(u, thickness, n0, dn) and BPM propagate!/backpropagate! --
 * src/optical_components/bulk_propagators/bpm.jl:1-74, :130-142, :235-321.
 */
FO_API int fo_bpm_create(fo_bpm* bpm, int nx, int ny, int batch, double dx, double dy,
                         const double* lambdas, int n_lambdas, double thickness, double n0,
                         int n_slices, int checkpoint_every, double cos_correction, int flags);
/*
 * AS_BPM with the propagators of fo_asprop_create_ex: `options` selects the paraxial
 * and the tilted kernel (no filter), and the dn phase of field b uses
 * kdz_b = 2 pi dz / (cos(theta_x,b) cos(theta_y,b)) from the field's tilts.
 * Replaces: AS_BPM(u, thickness, n0, dn; paraxial) for fields with tilts --
 * bulk_propagators/bpm.jl:3-6 (compute_cos_correction), :54-74, :130-142.
 */
FO_API int fo_bpm_create_ex(fo_bpm* bpm, int nx, int ny, int batch, double dx, double dy,
                            const double* lambdas, int n_lambdas, double thickness, double n0,
                            int n_slices, int checkpoint_every, const fo_as_options* options, int flags);
FO_API int fo_bpm_destroy(fo_bpm bpm);
FO_API int fo_bpm_info(fo_bpm bpm, int* checkpoint_every, size_t* workspace_bytes);

/* dn: n_slices x ny x nx float (slice-major).  In place on u. */
FO_API int fo_bpm_forward(fo_bpm bpm, void* u, const float* dn, int direction, int save,
                          void* stream);

/* Adjoint in place on du; ddn (n_slices x ny x nx float) receives the gradient
 * when not NULL.  Requires a preceding fo_bpm_forward(save=1) on the same input. */
FO_API int fo_bpm_backward(fo_bpm bpm, void* du, const float* dn, float* ddn, int direction,
                           void* stream);

/* ---------------------------------------------------------------------- */
/* SquaredIntensityDifference                                              */
/* ---------------------------------------------------------------------- */

/*
 * I_t = sum of |u_b|^2 over the fields b with target_index[b] == t;
 * loss_t = sum (I_t - target_t)^2.  target_index (host array, batch entries,
 * values < n_targets) is copied into the metric.  NULL target_index maps field b
 * to slice b % n_targets (the broadcast of an (nx, ny, T) target over
 * (nx, ny, T, M) fields).
 * Replaces: SquaredIntensityDifference -- src/metrics/squared_intensity_difference.jl:58-90.
 */
FO_API int fo_sid_create(fo_sid* sid, int nx, int ny, int batch, int n_targets,
                         const int* target_index);
FO_API int fo_sid_destroy(fo_sid sid);

/* Computes the residuals I - target (kept in the metric for the pullback) and
 * writes loss[n_targets] (device float). */
FO_API int fo_sid_forward(fo_sid sid, const void* u, const float* target, float* loss,
                          void* stream);

/* du = 4 dc_t (I_t - target_t) u from the last fo_sid_forward on u; dc: device
 * float[n_targets] (NULL: all ones). */
FO_API int fo_sid_backward(fo_sid sid, const void* u, const float* dc, void* du, void* stream);

/*
 * The loss values of SquaredIntensityDifference (as fo_sid_forward's `loss`) for
 * callers that cannot allocate device memory: plug-ins whose host application
 * owns all device memory through its own pool allocator, or real-time loops
 * where an allocation's implicit synchronisation is not allowed.  It allocates
 * nothing: the per-block partial sums live in a fixed 256 KiB array compiled into
 * the library (1024 blocks x 64 slices), which every GPU that loads the library
 * holds until the process exits.  target_index is a device int[batch] (values
 * < n_targets); n_targets may not exceed FO_SID_NOALLOC_MAX_TARGETS, larger
 * values return FO_ERR_SHAPE.  The first call on a device looks the array's
 * device address up (cudaGetSymbolAddress), so make that first call before any
 * stream capture.  The address is kept for the life of the process, so a
 * cudaDeviceReset after that first call is not supported.  All calls share the
 * array: calls that overlap on the GPU (different streams, no ordering between
 * them) race and give wrong losses.
 * No counterpart in the reference (it allocates freely on the Julia side).
 */
#define FO_SID_NOALLOC_MAX_TARGETS 64
FO_API int fo_sid_loss_noalloc(const void* u, const float* target, const int* target_index, int n_targets,
                               int nx, int ny, int batch, float* loss, void* stream);

/*
 * SquaredFieldDifference against reference fields v of the same grid and batch:
 * c[b] = sum over the field's pixels of |u_b - v_b|^2 (device float[batch];
 * fixed-order sums), and the pull-back du = 2 dc[b] (u_b - v_b) (dc: device
 * float[batch], NULL: all ones).
 * Replaces: SquaredFieldDifference -- src/metrics/squared_field_difference.jl:35-61.
 */
typedef struct fo_sfd_s* fo_sfd;
FO_API int fo_sfd_create(fo_sfd* sfd, int nx, int ny, int batch);
FO_API int fo_sfd_forward(fo_sfd sfd, const void* u, const void* v, float* c, void* stream);
FO_API int fo_sfd_backward(fo_sfd sfd, const void* u, const void* v, const float* dc, void* du, void* stream);
FO_API int fo_sfd_destroy(fo_sfd sfd);

/*
 * fo_chain_withgradient_sid for SquaredFieldDifference against the reference fields v:
 * c[b] (device float[batch]) receives the per-field values and du the gradient of
 * sum_b dc[b] c[b] (dc: device float[batch], NULL: ones).  When the last slot is empty
 * and no probes are set, the forward sweep's last row pass, the metric, its pull-back
 * 2 dc_b (u_b - v_b) and the adjoint sweep's first row pass are one pass (4K + 1
 * passes); the gradients equal those of the separate calls bit for bit, and the values
 * c differ from fo_sfd_forward's only in the order of the per-field sums.  Neither u_in
 * nor v may alias u_out or du.
 * Replaces: Zygote.withgradient over the reference's rrules for a system ending in a
 * propagator with SquaredFieldDifference (src/metrics/squared_field_difference.jl:35-61)
 * as the loss.
 */
FO_API int fo_chain_withgradient_sfd(fo_chain chain, const void* u_in, void* u_out, void* du,
                                     const fo_mod* mods_fwd, const fo_mod* mods_bwd, int direction, fo_sfd sfd,
                                     const void* v, const float* dc, float* c, int flags, void* stream);

/* ---------------------------------------------------------------------- */
/* Optimiser and proximal operators                                        */
/* ---------------------------------------------------------------------- */

/*
 * One Fista step on n floats: t' = (1+sqrt(1+4t^2))/2, beta = (t-1)/t',
 * newdx = eta^2 dx - beta (x - xk), xk <- x, x -= newdx, t <- t'.  `eta` is the
 * value given to Fista(eta) (the rule stores eta^2); t_state is a device double
 * (initialise to 1), read and advanced on the stream, so the step can be
 * replayed from a CUDA graph.
 * Replaces: Fista -- src/OptimisersExt.jl:33-54 with Optimisers' subtract!.
 */
FO_API int fo_fista_step(float* x, float* xk, float* newdx, const float* dx, long long n,
                         double eta, double* t_state, void* stream);

/* fo_fista_step followed by x = clamp(x, lo, hi), in one pass over the arrays.
 * Replaces: ProxRule(Fista(eta), ClampProx(lo, hi)) -- src/OptimisersExt.jl:222-244 with
 * proximal_operators/clamp_prox.jl:35-37. */
FO_API int fo_fista_clamp_step(float* x, float* xk, float* newdx, const float* dx, long long n,
                               double eta, double* t_state, double lo, double hi, void* stream);

/* x = clamp(x, lo, hi).  Replaces ClampProx (proximal_operators/clamp_prox.jl:35-37). */
FO_API int fo_clamp(float* x, long long n, double lo, double hi, void* stream);

/* Soft threshold of every value towards c: c where |x - c| <= s, else x -+ s.  A
 * complex parameter is passed as its 2n floats (the reference shrinks the real and the
 * imaginary part separately, each towards c).
 * Replaces: IstaProx(s, c) -- proximal_operators/ista_prox.jl:1-56 with PointwiseProx
 * (pointwise_prox.jl:31-46). */
FO_API int fo_ista(float* x, long long n, double s, double c, void* stream);

/* x = max(x, 0).  Replaces: PositiveProx -- proximal_operators/positive_prox.jl:1-40. */
FO_API int fo_positive(float* x, long long n, void* stream);

/*
 * One step x <- x - newdx of a plain gradient rule, in FP32 with the rule's own
 * operation order (no fused multiply-adds):
 *   FO_RULE_DESCENT  : newdx = eta dx (state unused, may be NULL)
 *   FO_RULE_MOMENTUM : v = rho v + eta dx; newdx = v
 *   FO_RULE_NESTEROV : newdx = (-rho^2) v + ((1 + rho) eta) dx; v = rho v - eta dx
 * state is the velocity v (n floats, zero at init).  A complex parameter is passed as
 * its 2n floats.
 * Replaces: Descent / Momentum / Nesterov of Optimisers.jl 0.4 (the version the
 * reference's Project.toml pins), re-exported by the reference (src/OptimisersExt.jl:9)
 * and used with make_rules / ProxRule (OptimisersExt.jl:195-244).
 */
#define FO_RULE_DESCENT 0
#define FO_RULE_MOMENTUM 1
#define FO_RULE_NESTEROV 2
FO_API int fo_rule_step(float* x, float* state, const float* dx, long long n, int rule, double eta, double rho,
                        void* stream);

/*
 * TVProx(lambda, n_iter; isotropic, rule = Fista(eta)) on an ny x nx float
 * array (fo_tv_create_nd: 1- to 3-D), in place: n_iter dual Fista iterations with the reference's D / D^T
 * boundary handling and per-slice normalisation.  fo_tv_create_ex adds `tol`
 * (0: none): the iterations stop, before their dual update, once the largest change
 * of the primal iterate from the previous iteration is below tol (tested on the
 * device; the remaining launches do nothing, so the call stays graph-capturable).
 * Replaces: TVProx / TV_denoise! -- src/proximal_operators/tv_prox.jl:1-258.
 */
typedef struct fo_tv_s* fo_tv;
FO_API int fo_tv_create(fo_tv* tv, int nx, int ny, double lambda, int n_iter, int isotropic,
                        double eta);
FO_API int fo_tv_create_ex(fo_tv* tv, int nx, int ny, double lambda, int n_iter, int isotropic,
                           double eta, double tol);
/* The same on a 1-, 2- or 3-D array of dims[0] x dims[1] x dims[2] (x fastest), with
 * one dual slice per dimension (the reference's n-dimensional D / D^T). */
FO_API int fo_tv_create_nd(fo_tv* tv, int ndims, const int* dims, double lambda, int n_iter, int isotropic,
                           double eta, double tol);
FO_API int fo_tv_destroy(fo_tv tv);
FO_API int fo_tv_apply(fo_tv tv, float* x, void* stream);

/* ---------------------------------------------------------------------- */
/* CUDA graphs of whole iterations                                         */
/* ---------------------------------------------------------------------- */

/*
 * Stream-ordered copy of `bytes` between host and device memory, either
 * direction (the pointers decide).  With page-locked host memory it is
 * asynchronous and can be captured into a graph.  It lets a host without CUDA
 * bindings upload fields and read results back through this library.
 * No counterpart in the reference (Julia moves data with CuArray / Array).
 */
FO_API int fo_copy(void* dst, const void* src, size_t bytes, void* stream);

typedef struct fo_graph_s* fo_graph;
FO_API int fo_graph_begin(void* stream);
FO_API int fo_graph_end(void* stream, fo_graph* graph);
FO_API int fo_graph_launch(fo_graph graph, void* stream);
/* Number of kernel nodes in a captured graph. */
FO_API int fo_graph_info(fo_graph graph, int* kernel_nodes);
FO_API int fo_graph_destroy(fo_graph graph);

/* ---------------------------------------------------------------------- */
/* Overlap metrics: DotProduct and PowerCoupling                            */
/* ---------------------------------------------------------------------- */

/*
 * Against reference fields v (batch x ny x nx complex float, borrowed for DotProduct;
 * PowerCoupling keeps unit-power copies made at creation):
 *   mode_selective = 1: c[b] = dx dy sum_p u_b[p] conj(v_b[p])                 (batch values)
 *   mode_selective = 0: c[i + j batch] = dx dy sum_p conj(v_i[p]) u_j[p]       (batch^2 values,
 *                       the column-major v' u of the reference; batch <= 64)
 * DotProduct (power = 0) writes complex float c; PowerCoupling (power = 1) writes
 * float |c|^2.  fo_overlap_backward writes du = v g (du_j = sum_i v_i G[i + j batch] for
 * the matrix form) with g = dc (complex) or 2 dc c (dc real, c of the last forward).
 * Reductions run in a fixed order (deterministic).
 * Replaces: compute_metric / backpropagate_metric of DotProduct (metrics/dot_product.jl:47-100)
 * and PowerCoupling (metrics/power_coupling.jl:48-66).
 */
typedef struct fo_overlap_s* fo_overlap;
FO_API int fo_overlap_create(fo_overlap* ov, int nx, int ny, int batch, double dx, double dy, const void* v,
                             int mode_selective, int power);
FO_API int fo_overlap_forward(fo_overlap ov, const void* u, void* c, void* stream);
FO_API int fo_overlap_backward(fo_overlap ov, const void* dc, void* du, void* stream);
FO_API int fo_overlap_destroy(fo_overlap ov);

/* ---------------------------------------------------------------------- */
/* Ragged batch: many independent problems of different sizes, one launch  */
/* ---------------------------------------------------------------------- */

/*
 * One problem: Phase(phase) -> ASProp(z; n0) -> SquaredIntensityDifference(target)
 * on an n x n grid (n a power of two from 256 to 4096), one field.  fo_ragged_batch
 * computes, for every problem of the plan, the propagated field u_out, the loss
 * sum((|u_out|^2 - target)^2) and its gradient with respect to the phase, i.e.
 * forward + adjoint, in ONE persistent cooperative kernel launch (plus one
 * memset of its counters).  All pointers are device pointers bound at creation;
 * u_in is only read (it is the saved input of the phase) and must not alias u_out.
 * Replaces, batched over independent problems, Zygote.withgradient of
 * SquaredIntensityDifference over ScalarSource |> Phase |> ASProp
 * (modulators/phasemask.jl:90-150, freespace_propagators/angular_spectrum.jl:193-234,
 * metrics/squared_intensity_difference.jl:58-90, src/ChainRulesCoreExt.jl:21-111).
 */
typedef struct fo_ragged_s* fo_ragged_plan;
typedef struct {
  int n;
  double dx, dy;
  double lambda, z, n0; /* n0 <= 0 means 1 */
  const void* u_in;     /* complex float[n][n] */
  const float* phase;   /* float[n][n] */
  const float* target;  /* float[n][n] intensity target */
  void* u_out;          /* complex float[n][n] */
  float* grad_phase;    /* float[n][n] */
  float* loss;          /* float[1] */
} fo_ragged_problem;

FO_API int fo_ragged_create(fo_ragged_plan* plan, const fo_ragged_problem* problems, int count, int flags);
FO_API int fo_ragged_batch(fo_ragged_plan plan, void* stream);
/* CTAs of the persistent launch (one per SM) and the workspace the plan owns. */
FO_API int fo_ragged_info(fo_ragged_plan plan, int* grid_ctas, size_t* workspace_bytes);
/* Device time of the five passes of the last completed fo_ragged_batch (ms[5]: row,
 * column, row, adjoint column, row + loss sums), from %globaltimer stamps taken by
 * the first CTA after each grid barrier.  Synchronizes the device. */
FO_API int fo_ragged_pass_ms(fo_ragged_plan plan, double* ms);
FO_API int fo_ragged_destroy(fo_ragged_plan plan);

#ifdef __cplusplus
}
#endif

#endif /* FLUXOPTICS_GB300_H */
