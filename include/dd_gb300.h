/*
 * dd_gb300.h -- C ABI of the GB300-native pseudospectral RHS / timestepping
 * library (libdd_gb300.so).
 *
 * Conventions
 *  - Every entry point returns an int status (DD_OK = 0); dd_last_error()
 *    gives a message for the calling host thread's last failure.
 *  - All array arguments are DEVICE pointers owned by the caller; the library
 *    never allocates caller-visible memory.  Plans own only their small
 *    wavenumber and twiddle tables; scratch space is passed in by the caller
 *    (size from dd_plan_workspace_size).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    asynchronous with respect to the host.
 *  - Layouts are the reference's (dedalus/data_objects/representations.py:86-93):
 *      3D x-space float64 [z][y][x],  k-space complex128 [ky][kz][kx], kx < Nx/2+1
 *      2D x-space float64 [y][x],     k-space complex128 [kx][ky]
 *    complex128 is interleaved (re, im) doubles.
 *  - Transform sizes per axis: powers of two 8 .. 512, and 24, 48, 96, 192
 *    (3 x a power of two; FP64/FP32 arithmetic).
 */
#ifndef DD_GB300_H
#define DD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (mapped to Python exceptions by the host binding) */
#define DD_OK              0
#define DD_ERR_INVALID     1  /* bad argument (null pointer, bad size)      -> ValueError */
#define DD_ERR_UNSUPPORTED 2  /* shape / option not supported               -> NotImplementedError */
#define DD_ERR_CUDA        3  /* CUDA runtime error                         -> RuntimeError */
#define DD_ERR_TIMEOUT     4  /* a bounded device wait expired              -> TimeoutError */
#define DD_ERR_WORKSPACE   5  /* workspace too small                        -> ValueError */

#define DD_FP64 0
#define DD_FP32 1
#define DD_DF64 2  /* double-float: transforms on FP32 pipes, ~48-bit significands */

typedef struct dd_plan dd_plan;

/* Library version (major*10000 + minor*100 + patch). */
int dd_version(void);
/* Message describing this host thread's most recent failure ("" if none). */
const char* dd_last_error(void);

/* ------------------------------------------------------- observability
 * Launch accounting and per-kernel device timing, the GPU analogue of the
 * reference's cumulative @timer (dedalus/utils/timer.py:29-65).
 * dd_launch_count: kernels launched by this library since load.
 * dd_timing_enable(1): bracket every launch with CUDA events on its stream;
 * dd_timing_report fills buf with "label count total_ms" lines (synchronises
 * the recorded events); dd_timing_reset clears the totals. */
long long dd_launch_count(void);
int dd_timing_enable(int on);
int dd_timing_reset(void);
int dd_timing_report(char* buf, size_t len);

/* ------------------------------------------------------------------ plans
 * One plan per grid geometry, the analogue of the reference's FFTW plan pair
 * (dedalus/utils/fftw/_fftw.pyx:246-309 rPlan, created in
 * representations.py:312-316).  xshape is (Nz, Ny, Nx) or (Ny, Nx).  k tables
 * are the reference's wavenumbers (representations.py:204-233) in k-layout
 * order: kx[Nx/2+1], ky[Ny], kz[Nz] (3D) or kx[Nx/2+1], ky[Ny] (2D), on the
 * host.  mx, my, mz give the largest kept |mode index| per axis after
 * dealiasing (representations.py:359-408): kept modes are 0..m and N-m..N-1.
 * Fails with DD_ERR_UNSUPPORTED for other sizes.
 */
int dd_plan_create(int ndim, const int64_t* xshape, const double* kx, const double* ky,
                   const double* kz, int mx, int my, int mz, dd_plan** out);
int dd_plan_destroy(dd_plan* plan);

/* Tile schedule of a pass group of this plan (which = 0: the y passes of the
 * fused 2D steps, dd_rhs2d / dd_rk2mid_step2d): variant 0 is the default,
 * 1 and 2 run the default tile's radix sequence on smaller tiles (bitwise the
 * same results, except against a single run of 64 or 128 points, whose
 * default is the small-tile schedule with its own radix sequence); dd_plan_get_schedule reports the current variant and how many this
 * plan's length offers (3 for 64, 128, 256, 512 points, else 1; a variant
 * the length lacks runs the default).  Set by the ensemble autotuner.  No
 * counterpart in the reference (FFTW chooses its own plans:
 * dedalus/utils/fftw/_fftw.pyx:246-309, flags FFTW_MEASURE). */
int dd_plan_set_schedule(dd_plan* plan, int which, int variant);
int dd_plan_get_schedule(const dd_plan* plan, int which, int* variant, int* count);

/* Scratch bytes needed by dd_fft_* for `nfield` fields at `precision`. */
int dd_plan_workspace_size(const dd_plan* plan, int nfield, int precision, size_t* bytes);

/* Forward transform x -> k of nfield fields: r2c, scaled by 1/N_total, then
 * 2/3 dealiasing (non-kept modes written as zeros).  Replaces
 * FourierRepresentation.forward = fwd_fftw + dealias (representations.py:318-345). */
int dd_fft_r2c(const dd_plan* plan, int nfield, const double* const* x, void* const* k,
               int precision, void* work, size_t work_bytes, void* stream);

/* Backward transform k -> x of nfield fields: c2r of the kept (dealiased)
 * modes, unnormalised.  The k arrays are read only; the reference's in-place
 * dealias before the transform is dd_dealias.  Replaces
 * FourierRepresentation.backward = dealias + rev_fftw (representations.py:323-357). */
int dd_fft_c2r(const dd_plan* plan, int nfield, const void* const* k, double* const* x,
               int precision, void* work, size_t work_bytes, void* stream);

/* Backward transform of one FP64 field, as dd_fft_c2r with nfield = 1, that
 * allocates nothing and takes no workspace.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory (an application
 * pool owns all of it, a per-call cudaMalloc and its device-wide
 * synchronisation are not allowed, or the caller's host language has no
 * device allocator).  Intermediates live in a 4 MiB static device buffer in
 * the library image (held on every GPU that loads the library): grids up to
 * 64^3 (3D) and 512^2 (2D), with or without 2/3 dealiasing (Nyquist modes are
 * never kept); larger ones return DD_ERR_UNSUPPORTED.  Each call looks the buffer
 * up on the current device (cudaGetSymbolAddress); the first call on a device
 * should come before any stream capture.  The plan must belong to the current
 * device (DD_ERR_INVALID otherwise).  All calls share the buffer: calls whose
 * GPU work overlaps race, so issue them in order on one stream. */
int dd_fft_c2r_noalloc(const dd_plan* plan, const void* k, double* x, void* stream);

/* *out (device double) = max over the ncomp grid-space arrays x[c] (n float64
 * values each, device) of x[c][i]^2: exact, deterministic, NaN-propagating.
 * Replaces VectorFieldBase.max_square (dedalus/data_objects/fields.py:153-157)
 * on one process, behind compute_dt / set_dtlist (physics.py:601-610,
 * 714-721, 830-836). */
int dd_max_square(int ncomp, const double* const* x, int64_t n, double* out, void* stream);

/* In-place 2/3 dealiasing of one k array.  Replaces dealias_cy_{2d,3d}.dealias_23
 * (dedalus/data_objects/dealias_cy_3d.pyx:13-37, dealias_cy_2d.pyx:59-78). */
int dd_dealias(const dd_plan* plan, void* k, void* stream);

/* Spectral derivative out = in * (1j * k_axis) of one k array (axis 0 = x,
 * 1 = y, 2 = z).  Replaces FourierRepresentation.deriv
 * (dedalus/data_objects/representations.py:419-425). */
int dd_deriv(const dd_plan* plan, int axis, const void* k_in, void* k_out, void* stream);

/* y = x * w (accumulate == 0) or y += x * w for n complex128 entries: the RK4
 * increment accumulation (dedalus/time_stepping/time_step.py:435, 452, 463, 474). */
int dd_scale_add(const void* x, void* y, double w, int accumulate, int64_t n, void* stream);

/* ------------------------------------------------------------ stage kernels
 * Same arguments and arithmetic as the reference's Cython kernels
 * (dedalus/time_stepping/forward_step_cy_3d.pyx:17-124 and
 * forward_step_cy_2d.pyx:21-120): contiguous complex128 arrays of n entries,
 * intfactor float64 (the reference passes -IF), output may alias start.
 * ndim selects the 2D or 3D Taylor branch.
 */
int dd_euler(const void* start, void* output, const void* deriv, double dt, int64_t n, void* stream);
int dd_etd1(int ndim, const void* start, void* output, const void* deriv, const double* intfactor,
            double dt, int64_t n, void* stream);
int dd_etd2rk1(int ndim, const void* start, void* output, const void* deriv1, const void* deriv2,
               const double* intfactor, double dt, int64_t n, void* stream);
int dd_etd2rk2(int ndim, const void* start, void* output, const void* deriv1, const void* deriv2,
               const double* intfactor, double dt, int64_t n, void* stream);

/* phi-function table for integer squared wavenumbers q = 0..qmax:
 * table[q] = {Z, f0(Z), f1(Z), f2(Z)} (4 doubles) with Z = -(nu q^vo) h, the
 * reference's intfactor*dt for k2 == q (physics.py:504-522), evaluated with
 * the stage kernels' arithmetic.  Used by the fused timesteppers. */
int dd_phi_table(int ndim, double nu, int viscosity_order, double h, int qmax, void* table, void* stream);

/* ------------------------------------------------------ fused 3D hydro
 * IncompressibleHydro.RHS (dedalus/physics/physics.py:527-599) for shear = 0,
 * Omega = None, no tracer and no forcing, computed as P[u x w] (rotational
 * form; equal on the kept modes to roundoff).  u and deriv are 3 component
 * k arrays (x, y, z order, full reference layout).  inv_k2 is an optional
 * device table 1/q for integer squared wavenumbers q (q = 0 -> 1); pass it
 * when every wavenumber is an integer (length-2 pi axes), else NULL.
 * zero_nonkept != 0 also writes zeros to the non-kept entries of deriv (the
 * reference zeroes deriv first, physics.py:140-142).  precision selects FP64
 * or FP32 transform/product arithmetic; the projection is FP64. */
int dd_hydro3d_workspace_size(const dd_plan* plan, int precision, size_t* bytes);
int dd_hydro3d_rhs(const dd_plan* plan, const void* const* u, void* const* deriv, const double* inv_k2,
                   int precision, int zero_nonkept, void* work, size_t work_bytes, void* stream);

/* One RK4 step of 3D hydro, in place on u.  Replaces RK4.do_advance
 * (dedalus/time_stepping/time_step.py:426-483), whose forward_step calls
 * undefined linear_step/intfac_step (time_step.py:209-218); the stage
 * definition is k1=N(y); y2=etd1(y,k1,dt/2); k2=N(y2); y3=etd1(y,k2,dt/2);
 * k3=N(y3); y4=etd1(y,k3,dt); k4=N(y4); y=etd1(y,k1/6+k2/3+k3/3+k4/6,dt).
 * tab_half / tab_full are dd_phi_table tables for h = dt/2 and h = dt (3D
 * variant) when inv_k2 is given; otherwise the phi functions are evaluated
 * per entry from nu and viscosity_order.  *nonkept_flag (host int) != 0 means
 * the state has energy outside the kept modes (see dd_any_nonkept); those
 * modes then decay as etd1(y, 0, dt), as in the reference. */
int dd_hydro3d_rk4_step(const dd_plan* plan, void* const* u, const double* inv_k2, const void* tab_half,
                        const void* tab_full, double nu, int viscosity_order, double dt, int precision,
                        int* nonkept_flag, void* work, size_t work_bytes, void* stream);

/* ------------------------------------------------------ fused 2D physics
 * physics 0 = IncompressibleHydro (physics.py:527-599), state (u_x, u_y);
 * physics 1 = BoussinesqHydro (physics.py:664-712), state (u_x, u_y, T) with
 * params = {g, alpha_t, beta, direction} (direction 0 = x, 1 = y; the
 * reference's default 'z' has no 2D component, physics.py:646, fields.py:148).
 * physics 2 / 3 = the same with the nonlinear terms in divergence form (the
 * momentum products u_x^2 - u_y^2, u_x u_y and the fluxes u_x T, u_y T: 2 + 2
 * and 3 + 4 transforms per RHS instead of 3 + 2 and 5 + 3), equal to physics
 * 0 / 1 to roundoff when every run's u is solenoidal (dd_divergence_sums2d).
 * Shear, rotation, tracer and forcing are not in these kernels.  A call covers
 * nrun independent runs of the plan's grid: run b's field c is at
 * state[c] + b * state_rs complex entries (state_rs = 0 and nrun = 1 for one
 * run).  dd_rhs2d writes the dealiased RHS into deriv (zero_nonkept != 0 also
 * zeroes the non-kept entries); dd_rk2mid_step2d advances the state in place
 * by one RK2mid step (time_step.py:275-309; euler/etd1/etd2rk2 with the 2D
 * Taylor branch), tab_half[c] / tab_full[c] being dd_phi_table(2, nu[c], vo, dt/2 or dt)
 * tables per state field when inv_k2 is given.  nonkept_flag: host int, 0
 * when the caller knows no run has energy outside the kept modes (the decay
 * of those modes is then skipped), or NULL to always treat them. */
int dd_rhs2d_workspace_size(const dd_plan* plan, int nrun, int precision, size_t* bytes);
int dd_rhs2d(const dd_plan* plan, int physics, const double* params, int nrun, const void* const* state,
             int64_t state_rs, void* const* deriv, int64_t deriv_rs, const double* inv_k2, int precision,
             int zero_nonkept, void* work, size_t work_bytes, void* stream);
int dd_rk2mid_step2d(const dd_plan* plan, int physics, const double* params, int nrun, void* const* state,
                     int64_t state_rs, const double* inv_k2, const void* const* tab_half,
                     const void* const* tab_full, const double* nu, int viscosity_order, double dt,
                     int precision, const int* nonkept_flag, void* work, size_t work_bytes, void* stream);

/* ------------------------------------------------------ fused 3D physics
 * physics 0 = IncompressibleHydro (state u_x, u_y, u_z; physics.py:527-599),
 * physics 1 = IncompressibleMHD (state u_x, u_y, u_z, B_x, B_y, B_z;
 * physics.py:770-819) with params = {rho0}, physics 2 = IncompressibleHydro
 * with the nonlinear term in divergence form (five products, 3 + 5 transforms
 * per RHS instead of 6 + 3; FP64 and FP32): equal to physics 0 to roundoff
 * when the state is solenoidal, which the caller checks (dd_divergence_sums);
 * physics 3 = IncompressibleMHD with the momentum term in divergence form
 * (five products of u u - B B / (4 pi rho0)) and the induction products u x B,
 * 6 + 8 transforms per RHS instead of 12 + 6: equal to physics 1 to roundoff
 * when u and B are solenoidal.
 * Shear, rotation, tracer and forcing are not in these kernels.  dd_rhs3d writes the dealiased RHS of every
 * state component into deriv (full layout); dd_rk4_step3d advances the state
 * in place by one RK4 step (definition as for dd_hydro3d_rk4_step) with one
 * diffusivity per vector field, coeff = {nu} or {nu, eta}, and one pair of
 * dd_phi_table tables per vector field.  nonkept_flag: host int, or NULL to
 * always treat modes outside the kept set (they decay as etd1(y, 0, dt)). */
int dd_rhs3d_workspace_size(const dd_plan* plan, int physics, int precision, size_t* bytes);
int dd_rhs3d(const dd_plan* plan, int physics, const double* params, const void* const* state, void* const* deriv,
             const double* inv_k2, int precision, int zero_nonkept, void* work, size_t work_bytes, void* stream);
int dd_rk4_step3d(const dd_plan* plan, int physics, const double* params, void* const* state, const double* inv_k2,
                  const void* const* tab_half, const void* const* tab_full, const double* coeff,
                  int viscosity_order, double dt, int precision, const int* nonkept_flag, void* work,
                  size_t work_bytes, void* stream);

/* ---------------------------------------------------------- diagnostics
 * Volume averages in k-space with the reference's Hermitian weights (entries
 * with kx > 0 count twice; dedalus/analysis/volume_average.py:71-98), summed
 * in FP64 with compensated, deterministic reductions.  kind:
 *   0 energy 1/2 sum|u_c|^2 (ekin/emag, volume_average.py:109-118, 180-188)
 *   1 1/2 |curl u|^2, 3D (energy_dissipation = 2 nu x this, 254-265)
 *   2 2D enstrophy 1/2 |d_x u_y - d_y u_x|^2 (191-200)
 *   3 helicity Re(u . conj(curl u)), 3D
 *   4 mean square divergence |sum_i i k_i u_i|^2
 *   5 divergence_sum: unweighted sum |sum_i i k_i u_i| (288-295)
 *   6 |u|^2 of one component (ux2, uy2, temp2, ...)
 * out is a device double.  dd_spectrum bins power1d = norm sum_c |u_c|^2 x
 * 4 pi k^2 (3D) or 2 pi k (2D) by kbottom[i] <= |k| < ktop[i], skipping zero
 * power (analysis_set.py:778-815); bin sums and counts are device arrays and
 * dk = kbottom[1]. */
int dd_diag_workspace_size(const dd_plan* plan, int nbins, size_t* bytes);
int dd_volume_average(const dd_plan* plan, int kind, int ncomp, const void* const* comps, double* out, void* work,
                      size_t work_bytes, void* stream);
int dd_spectrum(const dd_plan* plan, int ncomp, const void* const* comps, double norm, int nbins, const double* kbottom,
                const double* ktop, double dk, double* out_sum, double* out_count, void* work, size_t work_bytes,
                void* stream);

/* out[0] = sum |k . u|^2, out[1] = sum |k|^2 |u|^2 over the kept modes of a
 * 3D velocity (3 full-layout k arrays); out is device memory [2], overwritten.
 * out[0] / out[1] is the squared relative divergence of the state. */
int dd_divergence_sums(const dd_plan* plan, const void* const* u, double* out, void* stream);
/* The same for nrun 2D velocities (u_x, u_y full-layout k arrays; run r at
 * offset r * run_stride complex entries), summed over all runs. */
int dd_divergence_sums2d(const dd_plan* plan, int nrun, const void* ux, const void* uy, int64_t run_stride,
                         double* out, void* stream);

/* Sets *dflag (device int) to 1 if any of the ncomp k arrays has a non-zero
 * entry outside the kept (dealiased) modes; does not clear it. */
int dd_any_nonkept(const dd_plan* plan, int ncomp, const void* const* k, int* dflag, void* stream);

/* ------------------------------------------------- learned subgrid closure
 * No counterpart in the reference: a 64^3 LES of IncompressibleHydro whose
 * RHS gains -P[d_j tau_ij], tau predicted pointwise by an MLP
 * 10 -> 64 -> 64 -> 6 (tanh) from the resolved velocity gradients
 * G[3 i + j] = d_j u_i and the filter width.  Weights are BF16 on the tensor
 * cores with FP32 accumulation, master weights FP32.
 *   params: FP32 [nparam] = W1[64][16], b1[64], W2[64][64], b2[64], W3[8][64], b3[8]
 *   wbf16:  BF16 [nbf16]  = W1[64][16], W2[64][64], W3[16][64] (rows 8..15 zero)
 *   norm:   FP32 [48] = in_mean[16], in_scale[16], out_mean[8], out_scale[8];
 *           input a = (feature_a - in_mean[a]) * in_scale[a] (features 0..8 =
 *           G, 9 = filter width), stress c = y_c * out_scale[c] + out_mean[c]
 *           in the order xx, yy, zz, xy, xz, yz.
 * Samples: X [n][16] BF16 (columns 10..15 zero), targets T [n][8] FP32
 * (columns 6, 7 ignored), raw [n][16] FP32 = G (0..8), width (9), tau (10..15).
 * All arrays are device memory. */
typedef struct dd_closure {
    const void* wbf16;
    const float* params;
    const float* norm;
    double delta;          /* filter width fed to input 9 */
    double band_lo;        /* closure-term weight w(|k|): 0 for |k| <= band_lo, */
    double band_hi;        /* 1 for |k| >= band_hi, linear between; band_hi <= 0: w = 1 */
    const double* shell_w; /* device table; when not NULL it replaces the band: w(|k|) is */
    int n_shell;           /* shell_w linearly interpolated at |k| (entry i at |k| = i), */
                           /* shell_w[n_shell - 1] beyond the table */
} dd_closure;

int dd_mlp_sizes(int* nparam, int* nbf16, int* nnorm, int* in_dim, int* out_dim);
/* Workspace of dd_mlp_grad for a batch of n samples. */
int dd_mlp_workspace_size(int64_t n, size_t* bytes);
/* wbf16 = BF16(params). */
int dd_mlp_pack(const float* params, void* wbf16, void* stream);
/* Y [n][8] = MLP(X). */
int dd_mlp_infer(const void* X, float* Y, int64_t n, const void* wbf16, const float* params, void* stream);
/* Gradient of L = sum_s sum_{c<6} (Y_sc - T_sc)^2 / (6 n_total) over samples
 * s < n (row idx[s] of X and T when idx is not NULL) into grad [nparam]
 * (overwritten), and the squared-error sum into loss[0] (if not NULL).
 * Deterministic: per-block partials reduced in a fixed order. */
int dd_mlp_grad(const void* X, const float* T, const int64_t* idx, int64_t n, int64_t n_total, const void* wbf16,
                const float* params, float* grad, float* loss, void* work, size_t work_bytes, void* stream);
/* One Adam step (step counts from 1) on params, then wbf16 = BF16(params). */
int dd_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1, float beta2,
                float eps, void* wbf16, void* stream);
/* raw -> normalised X, T. */
int dd_mlp_normalize(const float* raw, int64_t n, const float* norm, void* X, float* T, void* stream);

/* Training data from a DNS: out (6 FP64 grid-point fields) = u_i u_j in the
 * order xx, yy, zz, xy, xz, yz. */
int dd_les_products(int64_t npts, const double* const* u, double* const* out, void* stream);
/* Sharp spectral filter: copy the modes kept on grid dst (|m_i| <= M_i of dst)
 * from the full-layout complex128 arrays of grid src to those of dst and zero
 * the rest of dst.  Both grids 3D with the same box; dst's kept set must lie
 * inside src's. */
int dd_les_truncate3(const dd_plan* src, const dd_plan* dst, int nfield, const void* const* s, void* const* d,
                     void* stream);
/* Grid-point velocity gradients gx[3 i + j] = d_j u_i of the full-layout
 * velocity u (3 complex128 arrays); work as for dd_les_workspace_size. */
int dd_les_gradients(const dd_plan* plan, const void* const* u, double* const* gx, int precision, void* work,
                     size_t work_bytes, void* stream);
/* raw[p] = (g_0..8, delta, f_c - fr_c for c = xx, yy, zz, xy, xz, yz) per
 * grid point: g the gradients, f = filt(u_a u_b) the filtered DNS products and
 * fr = filt(ubar_a ubar_b) the filtered products of the filtered velocity
 * (all grid-point values on the LES grid). */
int dd_les_samples(int64_t npts, const double* const* g, const double* const* f, const double* const* fr,
                   double delta, float* raw, void* stream);
/* Spectral band weight in place on nfield full-layout complex128 arrays: kept
 * modes times w(|k|) (0 for |k| <= lo, 1 for |k| >= hi, linear between; w = 1
 * when hi <= 0), non-kept modes zeroed. */
int dd_les_band(const dd_plan* plan, int nfield, void* const* k, double lo, double hi, void* stream);
/* Grid-point subgrid stress predicted by the closure for velocity u. */
int dd_les_stress(const dd_plan* plan, const void* const* u, double* const* tau, const dd_closure* cl,
                  int precision, void* work, size_t work_bytes, void* stream);
/* Subgrid energy transfer per wavenumber shell: out[b] = sum over the modes
 * with round(|k|) = b of Re(conj(u_a) (-i k_j tau_ij)^_a), counted over the
 * full spectrum (kx > 0 columns twice), for the velocity spectra u (3 full-layout
 * k arrays) and the grid-point stresses tau (6 FP64 fields, order xx, yy, zz,
 * xy, xz, yz); modes beyond bin nbins - 1 are left out.  Deterministic (fixed
 * summation order).  out is device memory [nbins]. */
int dd_les_transfer(const dd_plan* plan, const void* const* u, const double* const* tau, int nbins, double* out,
                    void* work, size_t work_bytes, void* stream);
/* Workspace of dd_les_gradients, dd_les_stress, dd_les_transfer, dd_les_rhs3d and dd_les_rk4_step3d. */
int dd_les_workspace_size(const dd_plan* plan, int precision, size_t* bytes);
/* RHS of the closed LES: dd_rhs3d (physics 0) plus -P[d_j tau_ij]. */
int dd_les_rhs3d(const dd_plan* plan, const void* const* state, void* const* deriv, const double* inv_k2,
                 int precision, int zero_nonkept, const dd_closure* cl, void* work, size_t work_bytes, void* stream);
/* One RK4 step of the closed LES, as dd_rk4_step3d (physics 0) with the
 * closure term in every stage. */
int dd_les_rk4_step3d(const dd_plan* plan, void* const* state, const double* inv_k2, const void* const* tab_half,
                      const void* const* tab_full, const double* coeff, int viscosity_order, double dt, int precision,
                      const int* nonkept_flag, const dd_closure* cl, void* work, size_t work_bytes, void* stream);

/* ---- Shearing box (FourierShearRepresentation, representations.py:558-740) ----
 * FP64 transforms of a shearing-box component at time t.  kys is the
 * component's sheared, wrapped k['y'] (representations.py:627-643) as a device
 * table, [ky][kx] (Ny x Nx/2+1) in 3D, [kx][ky] in 2D; cut = 2/3 of the y
 * Nyquist wavenumber; pr = the phase rate S * kx * y of the x-transformed
 * rows (representations.py:604-611), [y][kx] (Ny x Nx/2+1).
 * Forward: x r2c, times exp(+i pr t), y (and z) DFTs, 1/N, then the 2/3 rule
 * on (kx, k_y(t), kz) -- fwd_fftw + dealias (representations.py:676-691).
 * Backward: the 2/3 rule applied to the input as read (the array is not
 * modified), y (and z) inverse DFTs, times exp(-i pr t), x c2r -- rev_fftw
 * (representations.py:693-704).  Lengths as dd_fft_r2c. */
int dd_shear_workspace_size(const dd_plan* plan, int nfield, size_t* bytes);
int dd_shear_r2c(const dd_plan* plan, int nfield, const double* const* x, void* const* k, const double* kys,
                 double cut, const double* pr, double t, void* work, size_t work_bytes, void* stream);
int dd_shear_c2r(const dd_plan* plan, int nfield, const void* const* k, double* const* x, const double* kys,
                 double cut, const double* pr, double t, void* work, size_t work_bytes, void* stream);
/* In-place 2/3 rule with the sheared k_y: dealias_cy_{2d,3d}.dealias_23 with a
 * full-shape ky (dealias_cy_3d.pyx:39-45, dealias_cy_2d.pyx:36-40). */
int dd_shear_dealias(const dd_plan* plan, int nfield, void* const* k, const double* kys, double cut, void* stream);
/* k_out = 1j * k_y(t) * k_in (representations.py:419-425 with the sheared k['y']). */
int dd_shear_deriv_y(const dd_plan* plan, const double* kys, const void* k_in, void* k_out, void* stream);
/* Elementwise helpers of the shearing-box / rotating right-hand sides, each
 * operation rounded as numpy's elementwise expressions are:
 * k-space: out (+)= (in / r) * w (mode 0; numpy's complex-by-real division,
 * a product with 1 / r) or (in * r) * w (mode 1), r real, n complex entries;
 * grid points: out (+)= (a * b) * w (b may be NULL: a * w), n doubles. */
int dd_kspace_real(int64_t n, const void* in, const double* r, double w, int mode, int accumulate, void* out,
                   void* stream);
int dd_xspace_fma(int64_t n, const double* a, const double* b, double w, int accumulate, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DD_GB300_H */
