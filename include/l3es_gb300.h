/*
 * l3es_gb300 — C ABI of the GB300 (sm_103a) pseudo-spectral DNS hot path.
 *
 * Drop-in boundary for the l3es call surface (tumaer/ql-les-data). The reference
 * is a Python/JAX package of closures; each entry point below replaces one of its
 * functions, cited as file:line inside that project. Host code (the Python drop-in
 * package, or any C/C++/ctypes caller) passes raw CUDA device pointers, sizes and a
 * cudaStream_t (as void*). No PyTorch or CUDA-runtime types appear in signatures.
 *
 * Conventions
 *   - Spectral fields use the reference layout: 3D u_hat (batch, 3, N, N, N/2+1),
 *     2D u_hat (batch, 3, N, N/2+1), complex64 (interleaved float re, im), i.e. the
 *     output of jnp.fft.rfftn(u, axes) (l3es/spectral_solver.py:206).
 *   - Physical fields are float32 (batch, 3, N, N, N) in 3D, (batch, 3, N, N, 1) in 2D.
 *   - Every call is asynchronous on `stream` and returns 0 or a negative L3ES_E*
 *     code; it never aborts the process. l3es_last_error() describes the last
 *     failure of the calling thread.
 *   - A plan is not re-entrant: use one plan per stream. The plan owns its
 *     twiddle tables and scratch memory (allocated in l3es_plan_create); arrays
 *     passed to the calls are owned by the caller.
 */
#ifndef L3ES_GB300_H
#define L3ES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define L3ES_OK 0
#define L3ES_EINVAL (-1)   /* bad argument (size, pointer, mode) */
#define L3ES_ECUDA (-2)    /* CUDA runtime error (launch, allocation) */
#define L3ES_ENOMEM (-3)   /* device allocation failed */
#define L3ES_ESTATE (-4)   /* call not valid for this plan */
#define L3ES_ETIMEOUT (-5) /* a kernel's bounded wait on its own bulk copies ran out */
#define L3ES_ENONFINITE (-6) /* a step produced NaN or infinite values (blow-up) */

#define L3ES_FORCING_NONE 0        /* forcing_type="none" */
#define L3ES_FORCING_EKIN_TOT 1    /* forcing_type="ekin_tot" (spectral_solver.py:82-112) */
#define L3ES_FORCING_CONST_POWER 2 /* extension: eps/(2 E_f) u_hat on 0<|k|^2<=kf^2 */

typedef struct l3es_plan l3es_plan;

/* Solver parameters of set_up_solver(N, nu, dim, case, dt, seed, ckp_N, kf,
 * e_kin_target, forcing_type) (l3es/spectral_solver.py:156-168) that the step needs. */
typedef struct l3es_plan_desc {
  int32_t dim;        /* 2 or 3 (fft_axes (1,2) or (1,2,3)) */
  int32_t n;          /* grid points per axis: 8, 16, 32, 64, 128, 256 or 512 */
  int32_t batch;      /* independent trajectories stepped together (reference: 1) */
  int32_t forcing;    /* L3ES_FORCING_* */
  int32_t kf;         /* forcing band 0 < |k|^2 <= kf^2 (init_fields.py:167-188) */
  int32_t kolm_k;     /* extension, 2D: f_x = kolm_amp sin(kolm_k y); 0 = off */
  double nu;          /* viscosity */
  double dt;          /* time step */
  double e_kin_init;  /* ekin_tot target E0 (spectral_solver.py:209), all trajectories */
  double eps_inj;     /* extension: constant-power injection rate */
  double drag;        /* extension: linear drag coefficient */
  double kolm_amp;    /* extension: Kolmogorov forcing amplitude */
  int32_t scheme;     /* L3ES_SCHEME_*: how the step treats the viscous term */
} l3es_plan_desc;

/* The reference's explicit RK4 (du -= nu k^2 u_hat, l3es/spectral_solver.py:59). */
#define L3ES_SCHEME_EXPLICIT 0
/* Extension: RK4 with the viscous term integrated exactly by the factor
 * exp(-nu k^2 t) (Lawson's integrating-factor RK4); fourth-order like the explicit
 * form, and stable for any nu k^2 dt. l3es_rhs still returns the full right-hand side;
 * the adjoint calls refuse plans with this scheme. */
#define L3ES_SCHEME_INTEGRATING_FACTOR 1

/* Builds the closures' constant state of rhs_wrapper / rk4_wrapper
 * (l3es/spectral_solver.py:27-48, :65-71): twiddle tables, dealias band, scratch. */
int l3es_plan_create(const l3es_plan_desc* desc, l3es_plan** out);

/* Releases the plan's device memory. */
int l3es_plan_destroy(l3es_plan* plan);

/* Waits for the device, then reports (and clears) the plan's device error flags set
 * since the last check: L3ES_ETIMEOUT if a kernel gave up a bounded wait on its own
 * bulk copies (that CTA stopped early, so the results of that call are invalid), else
 * L3ES_ENONFINITE if a step wrote a NaN or infinity into the state (blow-up; the
 * reference shows it only through its umax / dt_est log columns,
 * l3es/spectral_solver.py:318-324). */
int l3es_plan_check(l3es_plan* plan);

/* Self-test of the bounded waits used by the bulk-copy kernels: one CTA waits on a
 * barrier that nothing completes. Returns L3ES_ETIMEOUT when the wait gave up as
 * designed (about 200 ms; the context stays usable), L3ES_OK if it did not. */
int l3es_selftest_bounded_wait(void* stream);

/* Per-trajectory ekin_tot target E0 (host array of `batch` doubles);
 * the reference computes it once in set_up_solver (spectral_solver.py:209). */
int l3es_plan_set_e0(l3es_plan* plan, const double* e0_host, int32_t count);

/* Per-trajectory viscosities (host array of `batch` doubles); the plan starts with
 * desc->nu for every trajectory. */
int l3es_plan_set_nu(l3es_plan* plan, const double* nu_host, int32_t count);

/* Scratch bytes the plan holds on the device (for capacity planning). */
int64_t l3es_plan_workspace_bytes(const l3es_plan* plan);

/* Kernel schedule of the plan's step (no counterpart in the reference, whose XLA
 * compiler picks its own kernels, spectral_solver.py:130-153): four choices,
 *   [0] 3D: x passes by the persistent bulk-tensor-copy kernels (else one tile per CTA);
 *       2D: the step's x passes in 2-column tiles (else 8 columns per CTA),
 *   [1] y passes with the radix-8 schedule (else radix 16 from N = 128),
 *   [2] the half-axis line pass: 1 two-for-one for 64 <= N <= 256, 2 two-for-one with
 *       radix-16 line FFTs, 3 the same fed by bulk copies (2 and 3: N = 256 only),
 *       0 the packed half-length one,
 *   [3] the persistent bulk-copy band x pass (else one tile per CTA).
 * Every schedule computes the same step; only speed differs. */
int l3es_plan_get_schedule(const l3es_plan* plan, int32_t* sched4);
int l3es_plan_set_schedule(l3es_plan* plan, const int32_t* sched4);

/* Form of the explicit RK4 step (the reference's stage sequence,
 * spectral_solver.py:65-80, in every form; only memory traffic differs):
 *   0 one elementwise update of the whole spectrum per stage,
 *   1 the same, with modes outside the dealiased rows taking the closed form of their
 *     linear decay (no nonlinear or forcing term reaches them),
 *   2 the stage combination fused into the band x pass, in place on the band, and
 *     every other mode scaled by its closed form inside the next stage's x inverse (no
 *     elementwise pass).
 * Plans start with form 2 in 3D and form 1 in 2D (the 2D band pass has too few CTAs to
 * hide the fused epilogue's memory latency).
 * Forms 1 and 2 apply when the forcing lies inside the band (constant-power kf <= kd,
 * Kolmogorov wavenumber < kt); otherwise, and for the integrating-factor scheme, the
 * step takes form 0. */
int l3es_plan_get_step_form(const l3es_plan* plan, int32_t* form);
int l3es_plan_set_step_form(l3es_plan* plan, int32_t form);

/* Autotuner: times one RK4 step of the plan (its step form, on its own scratch) under
 * each schedule choice (one knob at a time) and keeps the fastest. cache_path
 * (nullable) names a text file of earlier results, one line per GPU model, dim, N,
 * batch and step form; a hit skips the timing, a miss appends the result.
 * Synchronises the stream; not while recording a graph. */
int l3es_plan_autotune(l3es_plan* plan, const char* cache_path, void* stream);

/* Diagnostics of the drivers, FP64 results on the device (per trajectory):
 * l3es_field_stats: out[4] = max|u_x|, max|u_y|, max|u_z|, 0.5 mean sum u^2 of a
 *   physical field (spectral_solver.py:318-319; comp_dt at :123-127 follows from the
 *   maxima: cfl / min_c(umax_c / dx + nu / dx^2));
 * l3es_dissipation: out[1] = nu <|curl u|^2> of irfftn(i k x u_hat)
 *   (utils.py:300-315), by Parseval on the half spectrum;
 * l3es_energy_spectrum: ek[N] shell sums of |u_hat / N^dim|^2 * mul_fac over shells
 *   int(|k| + 0.5), times 4 pi k^2 / (samples + eps) (utils.py:35-97). */
int l3es_field_stats(l3es_plan* plan, const float* u, double* out_dev, void* stream);
int l3es_dissipation(l3es_plan* plan, const void* u_hat, double nu, double* out_dev, void* stream);
int l3es_energy_spectrum(l3es_plan* plan, const void* u_hat, double mul_fac, double* ek_dev,
                         void* stream);

/* Per-launch CUDA-event timing of the plan's kernels (tracing; the reference
 * only wall-clocks whole steps, spectral_solver.py:310-313). enable=1 clears the
 * counters and records an event pair around every launch on the call's stream;
 * enable=0 stops recording. */
int l3es_plan_timing(l3es_plan* plan, int32_t enable);

/* Totals for one kernel kind since timing was enabled (waits for the recorded
 * launches): summed device time, launch count and summed algorithmic bytes
 * (logical reads + writes, the roofline numerator). */
int l3es_plan_kernel_stats(l3es_plan* plan, int32_t kind, double* total_ms, int64_t* launches,
                           double* algo_bytes);

/* Number of kernel kinds and their names (for l3es_plan_kernel_stats). */
int32_t l3es_kernel_kind_count(void);
const char* l3es_kernel_kind_name(int32_t kind);

/* nsteps calls of step_fn(u, u_hat) (l3es/spectral_solver.py:73-118), in place on
 * u_hat. u_out (nullable) receives irfftn(u_hat) after the last step (:114-116).
 * e_inj_dev (nullable, device, nsteps*batch doubles) receives the per-step
 * injection rate of ekin_tot forcing (:109), 0 otherwise.
 * The first RK stage evaluates u from u_hat instead of reading the caller's u;
 * irfftn(rfftn(u)) == u for real u, so the result is the same up to rounding. */
int l3es_step(l3es_plan* plan, void* u_hat, float* u_out, int32_t nsteps,
              double* e_inj_dev, void* stream);

/* l3es_step, and the kinetic energy 0.5 <|u|^2> of the final state into ke_dev (device,
 * batch doubles; the quantity of spectral_solver.py:318), from the same energy pass that
 * ekin_tot forcing makes anyway (after ekin_tot forcing: the rescaled state's energy),
 * so it costs at most one pass over u_hat and no separate call or launch sequence. */
int l3es_step_energy(l3es_plan* plan, void* u_hat, float* u_out, int32_t nsteps,
                     double* e_inj_dev, double* ke_dev, void* stream);

/* rhs_fn(u, u_hat, rk) (l3es/spectral_solver.py:50-60): du = P[dealias *
 * rfftn(u x curl u)] - nu k^2 u_hat (+ enabled extension terms), u from u_hat.
 * du: device, same shape as u_hat, must not alias it. */
int l3es_rhs(l3es_plan* plan, const void* u_hat, void* du, void* stream);

/* jnp.fft.rfftn(u, axes=fft_axes) of a real field (spectral_solver.py:206). */
int l3es_rfftn(l3es_plan* plan, const float* u, void* u_hat, void* stream);

/* jnp.fft.irfftn(u_hat, axes=fft_axes) (spectral_solver.py:52, :114). */
int l3es_irfftn(l3es_plan* plan, const void* u_hat, float* u, void* stream);

/* Kinetic energy 0.5 mean(sum u^2) of irfftn(u_hat), by Parseval in FP64
 * (spectral_solver.py:318, :94). out_dev: device, batch doubles. */
int l3es_kinetic_energy(l3es_plan* plan, const void* u_hat, double* out_dev, void* stream);

/* ---- particle layer: spectral coarsening, NUFFT interpolation, advection ---- */

typedef struct l3es_interp_plan l3es_interp_plan;

/* Interpolator of spectral_interpolator_wrapper(ckp_N, fft_axes, splits, backend)
 * (l3es/integrator.py:26-34) plus the coarse grid of spectral_filtering
 * (l3es/utils.py:100-138). n_fine: grid of the spectra passed to
 * l3es_interp_set_spectrum (0 = coarse fields only); ckp_n: 8, 16, 32, 64 or 128;
 * width: ES kernel width (4, 6 or 8; upsampling 2); np_max: particle capacity. */
int l3es_interp_plan_create(int32_t dim, int32_t n_fine, int32_t ckp_n, int32_t width,
                            int64_t np_max, l3es_interp_plan** out);
/* Batched interpolator (no counterpart in the reference, which runs one trajectory per
 * job): `batch` trajectories of the same sizes, np_max particles each. It serves
 * l3es_interp_set_spectrum with the fine spectra of a batched step plan ([batch][3][...],
 * contiguous) and l3es_interp with backend 0 (NUFFT) on positions / velocities laid out
 * [batch][np][dim] (np per trajectory), each kernel launched once for all trajectories;
 * its other calls return L3ES_EINVAL. Results equal those of one plan per trajectory. */
int l3es_interp_plan_create_batch(int32_t dim, int32_t n_fine, int32_t ckp_n, int32_t width,
                                  int64_t np_max, int32_t batch, l3es_interp_plan** out);
int l3es_interp_plan_destroy(l3es_interp_plan* plan);

/* Coarse spectrum of spectral_filtering(irfftn(u_hat), ckp_N) taken directly from
 * the fine half spectrum (no fine-grid FFT): modes k in [-c/2, c/2-1]^dim scaled
 * by (c/N)^dim, Hermitian-averaged like real(ifftn(.)) (utils.py:115-127). */
int l3es_interp_set_spectrum(l3es_interp_plan* plan, const void* u_hat_fine, void* stream);

/* Coarse spectrum from a coarse physical field (3, c, c, c) / (3, c, c, 1), i.e. the
 * np.fft.fftn(u) of interpolate_finufft / interpolate_dft (integrator.py:38, :65). */
int l3es_interp_set_field(l3es_interp_plan* plan, const float* u_coarse, void* stream);

/* The coarse physical field: spectral_filtering's output (utils.py:126-127),
 * float32 (3, c, c, c) / (3, c, c, 1). */
int l3es_interp_coarse_field(l3es_interp_plan* plan, float* u_coarse, void* stream);

/* Copy of the current coarse half spectrum (3, c, c, c/2+1) / (3, c, c/2+1). */
int l3es_interp_coarse_spectrum(l3es_interp_plan* plan, void* out, void* stream);

/* u_r[j] = Re sum_k Hhat(k) exp(i k.r_j) / c^dim at np particles r (float64,
 * (np, dim)), into u_r (float64, (np, dim)): interpolate_finufft (backend 0, type-2
 * NUFFT, integrator.py:36-60) or interpolate_dft (backend 1, exact, :62-91).
 * r_out (nullable): shift_fn(r, dt * u_r) (integrator.py:21-23, combined.py:199). */
int l3es_interp(l3es_interp_plan* plan, const double* r, int64_t np, double* u_r,
                int32_t backend, double dt, double* r_out, void* stream);

/* Extension: particle advection by classical RK4 instead of the reference's explicit
 * Euler step (shift_fn(r, dt * u_r), integrator.py:21-23, combined.py:199), through the
 * plan's current coarse field held fixed over the step: four interpolations (backend as
 * in l3es_interp) at r, r + dt/2 v1, r + dt/2 v2, r + dt v3 (stage positions wrapped
 * into the box), r_out = (r + dt/6 (v1 + 2 v2 + 2 v3 + v4)) mod 2 pi. u_r receives v1,
 * the velocity at r (what l3es_interp returns). r, u_r and r_out must be separate. */
int l3es_interp_advect_rk4(l3es_interp_plan* plan, const double* r, int64_t np, double* u_r,
                           int32_t backend, double dt, double* r_out, void* stream);

/* Reverse mode of the particle interpolation: the reference differentiates
 * interpolate_finufft / interpolate_dft (integrator.py:36-91) after
 * spectral_filtering (utils.py:100-138) with jax.grad; here, for the velocities u_r of
 * l3es_interp_set_spectrum + l3es_interp at fixed positions r, and a cotangent
 * lam = dL/du_r (float64, (np, dim)), grad_fine receives dL/du_hat_fine (complex64,
 * the fine spectrum's shape, overwritten; convention of the adjoint calls below).
 * backend 0: the adjoint of the NUFFT (type-1 spread with the ES kernel, forward FFT of
 * the upsampled grid, deconvolution); 1: of the exact DFT. The plan needs n_fine > 0;
 * its coarse spectrum is not changed. */
int l3es_interp_vjp(l3es_interp_plan* plan, const double* r, int64_t np, const double* lam,
                    int32_t backend, void* grad_fine, void* stream);

/* Allocation-free form of l3es_interp_set_spectrum + l3es_interp(backend dft): no
 * counterpart in the reference. For hosts that cannot let a library allocate
 * device memory (e.g. a JAX/XLA FFI custom call, whose device memory belongs to
 * XLA's preallocated pool). Coarsens the fine half spectrum u_hat_fine (N =
 * n_fine) to ckp_N and evaluates the exact spectral interpolation at np particles
 * r (float64, (np, dim)) into u_r (float64, (np, dim)). Its one scratch buffer is a
 * fixed 417,792-byte array inside the library: ckp_N <= 32 in 3D, <= 64 in 2D,
 * larger sizes return L3ES_EINVAL, and so does np above 128 (2^31 - 1). Calls share
 * that array, so calls that overlap on the GPU race. Every call outside stream
 * capture looks up the array's device address on the current device; a call on a
 * capturing stream reuses the address of the last uncaptured call there, so make one
 * call per device before any capture. CUDA loads device code lazily: the first call
 * on a device loads the library's module and with it the array, so a host whose
 * device memory is spoken for makes that first (warm-up) call before handing the
 * device to its own pool, or sets CUDA_MODULE_LOADING=EAGER. */
int l3es_interp_dft_noalloc(int32_t dim, int32_t n_fine, int32_t ckp_n, const void* u_hat_fine,
                            const double* r, int64_t np, double* u_r, void* stream);

/* Particle velocities to the plan's coarse grid by the exact DFT of ur_to_u_dft_wrapper
 * (l3es/turbulence.py:299-339): S(k) = sum_j u_r[j] exp(-i k.r_j) on the full c^dim
 * grid, u_grid = real(ifftn(S)), float32 (3, c, c, c) / (3, c, c) (third component
 * zero in 2D). r, u_r: float64 (np, dim). */
int l3es_interp_particles_to_grid(l3es_interp_plan* plan, const double* r, const double* u_r,
                                  int64_t np, float* u_grid, void* stream);

/* shift_fn(r, scale * dr) = (r + scale * dr) mod box, elementwise over n doubles
 * (l3es/integrator.py:21-23). */
int l3es_shift(const double* r, const double* dr, int64_t n, double scale, double box,
               double* out, void* stream);

/* ---- Reverse mode (gradients through the RK4 step) ----
 * The reference obtains these derivatives with jax.grad of its step
 * (l3es/spectral_solver.py:50-80); here they are hand-written vector-Jacobian
 * products. Gradients of a real loss L with respect to a complex64 half spectrum z
 * use the convention dL/dRe z + i dL/dIm z (PyTorch's), i.e.
 * dL = Re sum(conj(grad) dz) over the stored entries. Supported forcings: none,
 * const_power (with drag and the Kolmogorov term) and ekin_tot (the kinetic-energy
 * rescaling after each step, spectral_solver.py:82-112, is differentiated: its adjoint
 * recomputes the step's last stage); plans with L3ES_SCHEME_INTEGRATING_FACTOR return
 * L3ES_EINVAL. The first call allocates the plan's adjoint workspace (16 spectra of the
 * plan's size); l3es_plan_adjoint_prepare does it ahead of time (before any capture). */
int l3es_plan_adjoint_prepare(l3es_plan* plan);

/* out = (d rhs / d u_hat)^T g at u_hat (the adjoint of l3es_rhs). */
int l3es_rhs_vjp(l3es_plan* plan, const void* u_hat, const void* g, void* out, void* stream);

/* One step backwards: lam holds dL/du_hat_{n+1} on entry and dL/du_hat_n on return,
 * u_hat_n is the state at the start of the step (the caller's checkpoint; not
 * modified). The inner RK4 stages are recomputed from it. */
int l3es_adjoint_step(l3es_plan* plan, const void* u_hat_n, void* lam, void* stream);

/* Loss on the plan's coarse grid, L = mean((spectral_filtering(irfftn(u_hat_fine), c)
 * - target)^2) over the dim velocity components (utils.py:100-138 for the
 * coarsening), into loss_dev (one double), and, when grad != NULL, dL/du_hat_fine
 * (complex64, the fine spectrum's shape). target: float32 (dim, c, c[, c]). The plan
 * must have been created with n_fine > 0. */
int l3es_interp_coarse_mse(l3es_interp_plan* plan, const void* u_hat_fine, const float* target,
                           double* loss_dev, void* grad, void* stream);

/* ---- SPH particle relaxation and density ----
 * Replaces the JAX-SPH neighbour list + quintic kernel + Tait EoS code of
 * l3es/relax.py:16-178 (relax_wrapper -> loop_body, sph_body) and l3es/utils.py:169-218
 * (rho_computer). A plan is made for n particles per axis at rest in the periodic box
 * [0, box)^dim: spacing dx = box / n, mass dx^dim, reference density 1, quintic kernel
 * of smoothing length dx and cutoff 3 dx, pressure p = p_ref (rho - 1) with
 * p_ref = (10 u_ref)^2. Positions, velocities and outputs are float64 (np, dim) device
 * arrays; np <= np_max. Positions are wrapped into the box before use. Outputs depend
 * only on the inputs (fixed neighbour order), not on the launch. */
typedef struct l3es_sph_plan l3es_sph_plan;
int l3es_sph_plan_create(int32_t dim, int32_t n, double box, int64_t np_max, l3es_sph_plan** out);
int l3es_sph_plan_destroy(l3es_sph_plan* plan);

/* rho_computer(n, dim, box)(r): rho[j] = dx^dim sum_{|r_jk| < 3 dx} W(|r_jk|), the
 * particle itself included (utils.py:205-216). rho: float64 (np,). */
int l3es_sph_density(l3es_sph_plan* plan, const double* r, int64_t np, double* rho, void* stream);

/* relax_wrapper(n, dim, box, is_physical, u_ref) loop_body(r) (relax.py:73-120): pressure
 * plus half the transport-velocity acceleration, in physical units (the reference's
 * non-dimensional mode returns the same values). */
int l3es_sph_relax_acceleration(l3es_sph_plan* plan, const double* r, int64_t np, double u_ref,
                                double* acc, void* stream);

/* relax_wrapper(...) sph_body(r, u) (relax.py:122-176): the pressure, viscous (eta = 1)
 * and transport-velocity accelerations as three (np, dim) arrays. */
int l3es_sph_forces(l3es_sph_plan* plan, const double* r, const double* u, int64_t np, double u_ref,
                    double* acc_p, double* acc_visc, double* acc_tvf, void* stream);

/* The combined loop's relaxation step (combined.py:132-142), fused:
 *   r_temp = shift(r0, dt u_r); a = loop_body(r_temp);
 *   r_temp = shift(r_temp, (relax_dt_factor dt)^2 a);
 *   u_out = periodic_displacement(r_temp, r0) / dt      (minimum image)
 * and, when r_out != NULL, the loop's advection r_out = shift(r0, dt u_out)
 * (combined.py:199). Outputs must not alias the inputs. */
int l3es_sph_relax_velocity(l3es_sph_plan* plan, const double* r0, const double* u_r, int64_t np,
                            double dt, double relax_dt_factor, double u_ref, double* u_out,
                            double* r_out, void* stream);

/* ---- CUDA graphs: record library calls once, replay them as one launch ----
 * No counterpart in the reference (its step is one XLA executable per trajectory,
 * spectral_solver.py:130-153). l3es_graph_begin returns a capturing stream; l3es_step,
 * l3es_rhs, l3es_interp*, l3es_shift and the diagnostics called with that stream are
 * recorded, not run (plan creation, l3es_plan_set_*, kernel timing and
 * l3es_interp_dft_noalloc's first call must happen before); l3es_graph_end turns the
 * recording into a graph that l3es_graph_launch runs on any stream, with the device
 * pointers it was recorded with. */
typedef struct l3es_graph l3es_graph;
int l3es_graph_begin(void** capture_stream);
int l3es_graph_end(void* capture_stream, l3es_graph** out);

/* Branches of a recording (no counterpart in the reference): l3es_graph_fork opens a
 * stream that joins the recording of capture_stream (or of one of its branches); calls
 * given it depend on what that stream had recorded so far and run concurrently with
 * everything recorded elsewhere until l3es_graph_join, after which the capturing
 * stream's later calls wait for the branch. Every fork must be joined before
 * l3es_graph_end, which releases the branch streams. Trajectories of different grid
 * sizes recorded on separate branches execute side by side in one graph launch. */
int l3es_graph_fork(void* capture_stream, void** branch_stream);
int l3es_graph_join(void* capture_stream, void* branch_stream);
int l3es_graph_launch(l3es_graph* graph, void* stream);
int l3es_graph_destroy(l3es_graph* graph);

/* Last error message of the calling thread ("" if none). */
const char* l3es_last_error(void);

/* Library version string. */
const char* l3es_version(void);

#ifdef __cplusplus
}
#endif

#endif /* L3ES_GB300_H */
