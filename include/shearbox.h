/*
 * shearbox.h -- C-ABI of the GB300 shearing-box RK3 time stepper.
 *
 * Drop-in boundary for the time step of hiiragiyua/shear_nnf (r1745).  The
 * reference has no plugin or FFI layer; its boundary is the Fortran routine
 *     cross(vor,phi,u00,w00,hv,hg,phiwk,vorwk,dvordy,rhvc1,rhvc2,rhgc1,rhgc2,chwk)
 * (cross.f90:3-4), called from disk3d (main.f90:279-280), calc_dns_disk3d
 * (gmres_shear.f90:3103-3104) and shoot_shear.f90:527, with its parameters in
 * modules ctes / running / bcs (mod.f90:1-130).  The entry points below are what
 * an ISO_C_BINDING interface of that routine binds (the Fortran module
 * include/shearbox_c.f90 declares them).
 *
 * Conventions
 *   - every function returns 0 on success and a positive error code otherwise;
 *     sb_last_error() describes the last failure of the calling thread.  Nothing
 *     in the library stops the process (the reference's `stop` statements become
 *     error codes or status flags).
 *   - state arrays use the reference pencil layout: vor/phi are
 *     complex(0:my1, 0:mx1, 0:mz1) stored as interleaved (re, im) doubles, y
 *     fastest (cross.f90:32-33, the `buffsize` arrays of main.f90:67 with one
 *     rank); u00/w00 are real(0:my1).  Host memory is caller-owned and copied;
 *     device memory is owned by the handle.
 *   - a handle holds `batch` independent boxes of one grid; it is not reentrant
 *     and owns one CUDA stream.  No CPU fallback exists: creation fails if no
 *     GPU is present.
 */
#ifndef SHEARBOX_H
#define SHEARBOX_H
#ifdef __cplusplus
extern "C" {
#endif

#define SB_TRACE_RECORD 24
#define SB_TRACE_RECORD_T 29   /* with the temperature (crosst) */

/* Run parameters.  Mirrors hre2.dat records 1, 2 and 4 as read by initcr
 * (initcr.f90:54-135) plus the run options of cross (running module,
 * mod.f90:54-81).  fixed_dt > 0 selects a constant step in place of the CFL
 * rule (the reference hard-codes ifix_dt=0, cross.f90:87,1608-1611). */
typedef struct sb_params {
  int mgalx, my, mgalz;        /* physical grid */
  double Re, alp, Ly, gam;     /* 1/nu, 2pi/Lx, Ly, 2pi/Lz */
  double s, chi, CFL;          /* shear rate, rotation, CFL number */
  double vbulk;                /* v of the (0,0) mode (cross.f90:1276) */
  double fixed_dt;             /* > 0: constant Delta t */
  int readflag;                /* 0: initial umax floor as for a created i.c. */
  double uprim;                /* hre2.dat uprime (used with readflag=0, s=0) */
  int nhist;                   /* UNER statistics every nhist steps */
  double etime, dumptime, dtimag; /* end time, dump time and interval */
  int keep_laminar;            /* 1: no stop on laminarisation (v_rms/Lz < 1e-5,
                                  cross.f90:2106-2115); the flag is still set */
  int les;                     /* iuse_LES: Smagorinsky eddy viscosity
                                  (cross.f90:1291-1406, hre3.dat keyword iuse_LES) */
  int les_visc;                /* iadd_visc: keep the molecular viscosity with the model */
  double cs;                   /* Cles, Smagorinsky constant; filter width
                                  (dx*dy*dz)^(1/3) (initcr.f90:510) */
  int ydeal;                   /* iydealiasing: 0 none (default), 3 compact y-filter
                                  of the state at every substep (cross.f90:214-227,
                                  476-490; filter_shear_hepta.f90:21-148) */
  int temperature;             /* itemperature: 1 steps the Boussinesq scalar tb of
                                  crosst (crosst.f90:3-1310) with sb_crosst or
                                  sb_set_temperature + sb_step */
  double fkappa, bym, gbeta;   /* its diffusivity, mean gradient d(Tbar)/dy and
                                  buoyancy factor (hre3.dat keyword itemperature,
                                  initcr.f90:1996-2011) */
  int damping;                 /* iadd_damping: 1 adds the window damping
                                  -damp_up Hw(y) u00 to the mean forcing rf0u
                                  (add_damping, operators.f90:42-84;
                                  cross.f90:625-626, crosst.f90:694-695) */
  double damp_up, damp_aa;     /* its permeability and half width / Lz
                                  (initcr.f90:2128) */
  int force;                   /* iadd_force: 1 or 2 adds the one- or two-pair
                                  streamwise-roll force to hv(kx=0, kz=1)
                                  (add_force, operators.f90:1-40), -1 the
                                  inertial force xforce to rf0u (cross.f90:610-624,
                                  crosst.f90:680-693) */
  double force_roll, xforce;   /* their amplitudes (initcr.f90:2103-2118) */
  int implicit_visc;           /* 1: viscous (and with the temperature, thermal)
                                  terms semi-implicit, the reference's explicit = 0
                                  (cross.f90:797-989, crosst.f90:916-1195; hre3.dat
                                  keyword explicit, initcr.f90:1976-1984): a
                                  Helmholtz solve (d2/dy2 - k^2 - Re/(beta_k dt))
                                  per line and substep, no viscous time-step limit
                                  (crosst: at most 6/CFL times it).  Needs les =
                                  ydeal = 0 and, with the temperature, fkappa > 0
                                  (error 2 otherwise). */
} sb_params;

/* Per-box status after sb_step (cross.f90 istop logic, 1683-1690, 2102-2115) */
typedef struct sb_status {
  int istop;        /* 1 if the run was asked to stop */
  int steps_done;   /* completed steps in the last call */
  int ntrace;       /* statistics records written in the last call */
  int flags;        /* 1 diverged (dt<1e-10), 2 NaN, 4 laminarised, 8 end time */
  double time, deltat, xoffb, xofft, cfl, cflv;
} sb_status;

typedef struct sb_handle sb_handle;

/* precision of sb_create: SB_FP64 computes everything in FP64 (the drop-in);
 * SB_MIXED stores the state in FP32 and runs the x/z transforms, the nonlinear
 * product and the RK3 arithmetic in FP32, while the compact y-solves, the
 * Helmholtz solve for v, the shear phases and the moving_frame remaps stay in
 * FP64.  The C-ABI takes and returns FP64 arrays in both cases. */
#define SB_FP64 0
#define SB_MIXED 1

/* Creates a handle for `batch` boxes: precomputes the compact-scheme
 * coefficients and factorisations (derivadas/prederiv1/prederiv2,
 * diffy_shear_hepta.f90:68-296,535-573), wavenumbers and CFL constants
 * (set_xyz_dy, initcr.f90:443-519) and allocates the device state.
 * Replaces initcr's set-up of the time step (initcr.f90:184-307). */
int sb_create(const sb_params *p, int batch, int precision, sb_handle **out);
int sb_destroy(sb_handle *h);

/* Per-box Reynolds number (ensembles); default p->Re. */
int sb_set_member_re(sb_handle *h, int member, double Re);

/* Per-box end time (the etime of running, mod.f90:58): a box stops at it,
 * with the last step shortened to land on it (cross.f90:1694-1711).  The
 * Newton/Arnoldi period map integrates every perturbation to time0 + T this way
 * (calc_dns_disk3d, gmres_shear.f90:2951-3120). */
int sb_set_member_etime(sb_handle *h, int member, double etime);

/* Copies one box's state in / out (what getfil / escru read and write,
 * readwrite.f90:72-447,1164-1402, minus the file). */
int sb_set_state(sb_handle *h, int member, const double *vor, const double *phi,
                 const double *u00, const double *w00, double time, double xoffb,
                 double xofft);
int sb_get_state(sb_handle *h, int member, double *vor, double *phi, double *u00,
                 double *w00, double *time, double *xoffb, double *xofft);

/* Temperature state of a box created with temperature = 1: tb in the pencil
 * layout of vor, tb00 real(0:my1) (the tb, tb00 arguments of crosst,
 * crosst.f90:3-5,47-49).  set_conj_t is applied to tb at the entry of each
 * sb_step call (crosst.f90:333-337). */
int sb_set_temperature(sb_handle *h, int member, const double *tb, const double *tb00);
int sb_get_temperature(sb_handle *h, int member, double *tb, double *tb00);

/* Advances every box by nsteps RK3 steps on the device, with the semantics of
 * one call of cross (cross.f90:336-1029): set_conj on entry, v from phi on the
 * first step, Delta t from the CFL (or fixed_dt) on every step, stop on
 * NaN / divergence / laminarisation / etime. */
int sb_step(sb_handle *h, int nsteps);
int sb_get_status(sb_handle *h, int member, sb_status *st);

/* Statistics records of the last sb_step (the .cfbin record of
 * cross.f90:2087): time, Deltat, uner(1:10), CFL, CFLv, umax(1:3), xoffb,
 * xofft, umax(0), uner2(1:4); SB_TRACE_RECORD doubles each, or
 * SB_TRACE_RECORD_T with the temperature, which appends tbmax, tner(1:4)
 * (crosst.f90:2456-2458). */
int sb_get_trace(sb_handle *h, int member, double *out, int max_records, int *nrec);

/* Drop-in for cross(): box 0's host state in, nstep steps, state out. */
int sb_cross(sb_handle *h, double *vor, double *phi, double *u00, double *w00, double *time,
             double *xoffb, double *xofft, int nstep, sb_status *st);

/* Drop-in for crosst() (crosst.f90:3-5, iadd_mode 5; the explicit branch, or
 * the semi-implicit one with implicit_visc): as sb_cross with the scalar tb and
 * its mean tb00; needs temperature = 1. */
int sb_crosst(sb_handle *h, double *vor, double *phi, double *u00, double *w00, double *tb,
              double *tb00, double *time, double *xoffb, double *xofft, int nstep,
              sb_status *st);

/* Statistics that hist accumulated over the last sb_step call (module
 * statistics, mod.f90:94-115; reset at the entry of every call,
 * cross.f90:139-155): per y plane the 23 quantities of stats and their
 * Delta t-weighted sums stats2 (hist 'f' and 'p', cross.f90:1830-1955,
 * 2038-2048; layout [my][23]), the kx-kz spectra spl and spl2 of uu, vv, ww,
 * uv, o1o1, o2o2, o3o3, o1o2 (cross.f90:1970-2014; layout [mz][nkx][8]), with
 * the temperature tstats [my][5] and splt [mz][nkx][4] (crosst.f90:2201-2205,
 * 2364-2374), the number of records nacum and their summed Delta t total_dt
 * (cross.f90:2070-2072).  The Delta t weights of a record are those of the
 * step before it, as in the reference.  Any pointer may be NULL. */
int sb_get_statistics(sb_handle *h, int member, double *stats, double *stats2, double *spec,
                      double *spec2, double *tstats, double *tspec, int *nacum,
                      double *total_dt);

/* The uner(1:10) and uner2(1:4) of the last statistics record of a member
 * (the quantities hist 'w' writes, cross.f90:2064-2118). */
int sb_stats(sb_handle *h, int member, double *uner, double *uner2);

/* Batched finite-difference products of the period map (matvec_dns_disk3d,
 * gmres_shear.f90:2666-2948, iopt_matvec 1 forward / 2 central):
 *   eps_q = eps_jacobi |x0| / |d_q|,  h_q = (x0 + eps_q d_q) - x0 (iuse_hej),
 *   out_q = (Phi_T(x0 + h_q) - Phi_T(x0)) / eps_q                 central = 0
 *   out_q = (Phi_T(x0 + h_q) - Phi_T(x0 - h_q)) / (2 eps_q)       central = 1
 * with Phi_T the integration from time0 (offsets xoffb, xofft) to time0 + T
 * (calc_dns_disk3d, gmres_shear.f90:2951-3120).  Vectors are states laid out
 * as [vor | phi | u00 | w00] (pencil layout, 4 nkx mz my + 2 my doubles),
 * norms plain 2-norms; dirs and out hold ndir such vectors.  Every perturbed
 * state is one member of the handle's batch, so a block of batch directions
 * is one batched integration.  The members' states and end times are
 * overwritten.  Not available for the temperature variant. */
int sb_jv_batch(sb_handle *h, const double *x0, double time0, double xoffb, double xofft,
                double T, const double *dirs, int ndir, double eps_jacobi, int central,
                double *out);

/* Device-resident unknown vectors of the Newton-Krylov and Arnoldi searches.
 * A packed vector is the unknown vector of `throwing` (gmres_shear.f90:
 * 2229-2426, iuse_fou_mode 2): u00/sca[0] (my), w00/sca[0] (my), then per y
 * plane j, per kz index k = 0..mz-1 and kx index i (skipping (0,0) and the
 * kx = 0 entries of negative kz, which set_conj restores) the four doubles
 * vor.re/sca[1], phi.re/sca[2], vor.im/sca[1], phi.im/sca[2]; its length is
 * sb_packed_length(h) = 2 my + 4 my (mz nkx - 1 - nz).  phi stands where the
 * reference throws v (a fixed invertible map per mode).  x is a DEVICE
 * pointer; the work is queued on the handle's stream.
 *   sb_set_state_packed  backthrowing + set_conj into a member, with its time
 *                        and image offsets (as sb_set_state does from host
 *                        arrays; the LES running maximum of nu_t restarts)
 *   sb_get_state_packed  throwing of a member's state, each mode multiplied by
 *                        exp(-i kx shiftx) exp(-i kz shiftz) (phase_shift_fou,
 *                        operators.f90:488-544) on the way
 * Not available for the temperature variant. */
long sb_packed_length(const sb_handle *h);
int sb_set_state_packed(sb_handle *h, int member, const double *x, const double sca[3],
                        double time, double xoffb, double xofft);
int sb_get_state_packed(sb_handle *h, int member, double *x, const double sca[3], double shiftx,
                        double shiftz);
/* d/ds of phase_shift_fou at s = 0 on a packed vector (device x, out; in place
 * allowed): every mode times -i kx (dir 0) or -i kz (dir 1), the mean profiles
 * zero -- the shift columns dG/ds and the phase-condition rows of the
 * relative-periodic-orbit system (gmres_shear.f90:2900-2934). */
int sb_packed_shift_tangent(sb_handle *h, const double *x, double *out, int dir);

/* A Krylov space on the device: `cols` FP64 vectors of n entries (columns
 * 256-byte aligned), replacing the rank-0 vector algebra of the reference's
 * GMRES and Arnoldi (dotp, vecadd, norm, gmres_shear.f90:3680-3919; the
 * Gram-Schmidt loops of gmres_k_shear, 1905-2207, and arnoldi_shear.f90:
 * 222-330).  Row ranges [r0, r1) select the entries an operation covers.
 * stream NULL gives the space its own stream; pass a handle's stream
 * (sb_get_stream) to order the space's work with that handle's.
 *   sb_kspace_gram       C[a][b] = <col a0+a, col b0+b>, m x p, row-major host
 *                        array; fixed-order reductions (bitwise reproducible)
 *   sb_kspace_update     col b0+b += alpha sum_a col a0+a C[a][b] (ranges
 *                        must not overlap; C host m x p row-major)
 *   sb_kspace_transform  cols b0..b0+p-1 <- (cols b0..) M, p <= 64, in place
 *   sb_kspace_combine    col dst = sum_k coef[k] col src[k], nsrc <= 8
 *   sb_kspace_perturb    col dst = x0 + ((x0 + e d) - x0) (the representable
 *                        step of matvec_dns_disk3d, iuse_hej)
 *   sb_kspace_fd         finite-difference product of order 1, 2 or 4 into
 *                        col dst from the columns g (2 or 4 of them): (g0-g1)/eps,
 *                        (g0-g1)/(2 eps), (8 (g0-g1) - (g2-g3))/(12 eps)
 *   sb_kspace_set/get    host <-> part of one column (synchronous)
 *   sb_kspace_col        device address of a column (NULL if out of range) */
typedef struct sb_kspace sb_kspace;
int sb_kspace_create(long n, int cols, void *stream, sb_kspace **out);
int sb_kspace_destroy(sb_kspace *ks);
double *sb_kspace_col(sb_kspace *ks, int col);
void *sb_kspace_stream(sb_kspace *ks);
int sb_kspace_sync(sb_kspace *ks);
int sb_kspace_gram(sb_kspace *ks, long r0, long r1, int a0, int m, int b0, int p, double *C);
int sb_kspace_update(sb_kspace *ks, long r0, long r1, int a0, int m, int b0, int p,
                     const double *C, double alpha);
int sb_kspace_transform(sb_kspace *ks, long r0, long r1, int b0, int p, const double *M);
int sb_kspace_combine(sb_kspace *ks, long r0, long r1, int dst, int nsrc, const int *src,
                      const double *coef);
int sb_kspace_perturb(sb_kspace *ks, long r0, long r1, int dst, int x0, int d, double e);
int sb_kspace_fd(sb_kspace *ks, long r0, long r1, int dst, int order, const int *g, double eps);
int sb_kspace_set(sb_kspace *ks, int col, long off, long len, const double *host);
int sb_kspace_get(sb_kspace *ks, int col, long off, long len, double *host);

/* Measurement hooks (no counterpart in the reference; used by the benchmark).
 * sb_launch_stage enqueues `count` launches of one kernel of substep rk on the
 * handle's stream: stage 1..3 the plane stages, 4 the per-box phase tables,
 * 5 and 6 the two y-line kernels of the split form, 12 the fused y-line kernel
 * (handles without temperature or y filter/dealiasing); with LES, 7..10 the four
 * LES plane kernels and 11 the LES y-line kernel; with implicit_visc, 13 the
 * factorisation of the substep's Helmholtz operators and 14 its y-line
 * kernel.  The launches act on the current device state, so a run that used
 * them must set the state again before stepping.
 * sb_fp64_peak measures the device's FP64 FMA throughput in TFLOP/s. */
int sb_launch_stage(sb_handle *h, int stage, int rk, int count);

/* Physical fields of a member's state as the post-processor convh5 writes
 * them (hvhg_uvwp, convh5.f90:650-933): mask bits 0..10 select u, v, w,
 * omega_x, omega_y, omega_z (the velocity with the laminar shear s*y and
 * omega_z with -s), Q and R of the velocity gradient tensor, Qs and Rs of the
 * strain tensor, Qw = |omega|^2/4.  out receives the selected fields in that
 * order, each [my][mgalz][mgalx] doubles.  The state is not changed. */
int sb_physical_fields(sb_handle *h, int member, unsigned mask, double *out);

/* Autotuner of the step's tiles (no counterpart in the reference): times the
 * tile candidates of plane stages 1-3 on the handle's current state -- kx
 * columns per block of stages 1 and 3 (4 or 8), threads per block of stage 2
 * (the default or twice it) -- and the y-line tile, 1, 2 or 3 warps per line
 * solve (segments of the banded rows solved at once; each choice has its own
 * factor tables) in either form of the y-line stage (below), then the side
 * branch mask (sb_set_side_branch) on that tile, keeps the fastest and
 * re-captures the step graph.  choice (may be NULL) receives cb1, cb3, t2;
 * sb_get_tuning gives cb1, cb3, t2 and the warps per line solve.  The state
 * itself is not changed; call it after sb_set_state and before sb_step.
 * sb_set_line_segments sets the warps per line solve directly (1..3; my - 3 >=
 * 6 rows per segment).
 * sb_set_line_form chooses the y-line kernels of a substep: 1 (the default
 * where available) one fused kernel that takes each group of lines through all
 * its solves, 0 the split pair; form 1 needs a handle without temperature or y
 * filter/dealiasing (otherwise error 1, and such handles always run form 0).
 * sb_get_line_form gives the form the step graph uses (2 for a handle with
 * implicit_visc, whose substeps run the semi-implicit y-line kernel).  Both
 * forms compute the same step (to the last bits in FP64).
 * sb_set_side_branch chooses which side work of a substep the step graph runs
 * as a branch concurrent with the plane stages: bit 0 the spectra of a
 * statistics step (beside plane stages 1-2), bit 1 the per-box scalars and
 * phase tables (beside plane stage 3; handles with LES always run these in
 * order); a cleared bit runs that work on the main stream in order.  The
 * default is 3 and sb_autotune picks the fastest mask; every mask computes the
 * same step bit for bit.  sb_get_side_branch gives the mask in use. */
int sb_autotune(sb_handle *h, int *choice);
int sb_get_tuning(sb_handle *h, int *out);
int sb_set_line_segments(sb_handle *h, int nseg);
int sb_set_line_form(sb_handle *h, int form);
int sb_get_line_form(sb_handle *h, int *form);
int sb_set_side_branch(sb_handle *h, int mask);
int sb_get_side_branch(sb_handle *h, int *mask);
int sb_fp64_peak(sb_handle *h, double *tflops);

/* Standalone y-line operators on device-resident complex lines.  Line data is
 * [j][line]: element (line, j) is the complex at u + 2*(j*ldu + line).  shp/shm
 * (and k2) are HOST arrays with one complex (one real) entry per line: the
 * shear phases of the upper / lower periodic images, u(y+Ly) = shp*u(y) and
 * u(y-Ly) = shm*u(y).  A real line is a complex line with zero imaginary part
 * and shp = shm = 1.  The work is enqueued on `stream` (a cudaStream_t, 0 for
 * the legacy stream) and the call returns once it has completed.
 *   sb_op_derivyc   first (iord 1) or second (iord 2) derivative in y with the
 *                   compact heptadiagonal scheme: derivyc,
 *                   diffy_shear_hepta.f90:333-450 (ias=1 semantics).
 *   sb_op_lapcdy    solves (d2/dy2 - k2) p = u: lapcdy,
 *                   diffy_shear_hepta.f90:466-525.
 * Both allocate their scratch and factor tables with the stream-ordered
 * allocator and free them before returning. */
int sb_op_derivyc(int my, double Ly, int iord, int nlines, const double *u, long ldu, double *out,
                  long ldo, const double *shp, const double *shm, void *stream);
int sb_op_lapcdy(int my, double Ly, int nlines, const double *u, long ldu, double *out, long ldo,
                 const double *k2, const double *shp, const double *shm, void *stream);

/* Compact y-filter of device lines, same layout and shp convention:
 * filterc (filter_shear_hepta.f90:104-148) with the fixed coefficients of
 * prefilter (:55-73), 9-point right-hand side over the cyclic heptadiagonal
 * left-hand side; the lower image uses conj(shp) as matvecNcyclic does
 * (diffy_shear_hepta.f90:978).  Allocates its scratch like sb_op_derivyc. */
int sb_op_filterc(int my, int nlines, const double *u, long ldu, double *out, long ldo,
                  const double *shp, void *stream);

/* y-line transforms in place on device lines (FFTW conventions; forward,
 * iopt < 0, scaled by 1/my; backward, iopt > 0, unscaled), my in
 * {32, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384}:
 *   sb_op_cfty  complex lines, element (line, j) at c + 2*(j*ldc + line):
 *               cfty, cftdoublew.F:151-201
 *   sb_op_rfty  real lines of my + 2 rows, element (line, j) at c + j*ldc + line;
 *               forward leaves the half spectrum packed as (re, im) pairs of
 *               modes 0..my/2 in rows 0..my+1, backward reads it and zeroes
 *               rows my, my+1: rfty, rftdoublew.F:133-158 */
int sb_op_cfty(int my, int nlines, double *c, long ldc, int iopt, void *stream);
int sb_op_rfty(int my, int nlines, double *c, long ldc, int iopt, void *stream);

/* Allocation-free variant of sb_op_derivyc (no counterpart in the reference).
 * For callers that must not allocate device memory where they need the
 * derivative -- e.g. an application whose device memory is all handed to its
 * own pool, or a loop that must not pay the synchronisation an allocation can
 * cause.  Same arguments and results as sb_op_derivyc; it calls no cudaMalloc,
 * cudaFree or allocating library routine.  Its scratch is one fixed device
 * array of the library (about 9.5 MB, held on every GPU that loads the library
 * until the process exits), limited to nlines <= SB_NOALLOC_LINES and
 * my * (2*nlines rounded up to a multiple of 32) <= SB_NOALLOC_YBUF doubles;
 * larger requests return error 6 with a message.  Every call looks up the
 * array's address in the current device's context (cudaGetSymbolAddress, no
 * allocation) and returns after its stream has finished the work.  Every call
 * overwrites the whole part of the array it uses, so nothing carries over
 * between calls, but all calls share the one array: calls that overlap on the
 * GPU (other streams, other host threads) race and must be serialised by the
 * caller. */
#define SB_NOALLOC_LINES 32768
#define SB_NOALLOC_YBUF (1L << 20)
int sb_op_derivyc_noalloc(int my, double Ly, int iord, int nlines, const double *u, long ldu,
                          double *out, long ldo, const double *shp, const double *shm,
                          void *stream);

/* Restart files in the reference's binary layout (no GPU needed).
 * sb_write_restart writes the state (pencil layout, as sb_set_state takes it)
 * as escru does (readwrite.f90:1336-1398): Fortran unformatted sequential
 * records with 32-bit little-endian length markers -- grid, parameters, y,
 * offsets, u00/w00, one record per y plane (vor.re, phi.re, vor.im, phi.im for
 * every kz, kx), then the footer CFL/uprim/vbulk/xforce, irev/nopt/nparams,
 * the 9 switches and 13 parameters.
 * sb_read_restart reads one as getfil does (readwrite.f90:72-447): with p NULL
 * only *info is filled; otherwise the state is mapped on p's grid and set_conj
 * is applied:
 *   x, z   the common kx modes and the lowest positive and negative kz modes,
 *          zeros elsewhere; a changed alp rescales the image offsets by
 *          alp_file/alp, and a doubled alp with half the x points keeps the
 *          file's even kx modes (ihalf)
 *   y      my = file my: as read; my = file my / 2: every other plane
 *          (ihalfy); my = 3 or 5 file my: the box stacked in y, copy n shifted
 *          by exp(-i kx xofft n), offsets times 3 or 5 (ncopy_y); any other
 *          my > file my: a natural cubic spline in y per mode line through the
 *          file's planes and the wrapped first plane at Ly/2 (interp_y,
 *          readwrite.f90:707-771; needs the file's Ly); my < file my (not
 *          half): the first my planes, as getfil reads them
 *   scale  a changed gam rescales u00, w00 by gam_file/gam, phi by
 *          gam/gam_file and (without LES) vor by (gam_file/gam) sqrt(Re/Re_file);
 *          a changed Re alone rescales vor by sqrt(Re/Re_file) (without LES and
 *          unless flags has SB_RESTART_KEEP_VOR, as the Newton drivers read)
 * The offsets of the mapped state are info->run_xoffb/run_xofft (info->xoffb/
 * xofft are the file's); info->ymap says which y mapping ran (0 as read,
 * 1 half, 2 stacked, 3 spline).  Errors: 7 I/O, 8 malformed file, 9
 * unsupported grid change (x and y together, alp and my together, a spline
 * with a different Ly); message in sb_last_error. */
#define SB_RESTART_MAXOPT 32
typedef struct sb_restart_info {
  int mgalx, my, mgalz, numerop;         /* record 1 */
  double time, Re, alp, Ly, gam, s, chi; /* record 2 (Ly = stored Ly/pi times pi) */
  int mx, mye, mz;
  double xoffb, xofft, zoffb, zofft;     /* record 4 */
  double CFL, uprim, vbulk, xforce;      /* footer */
  int has_footer, irev, nopt, nparams;
  int options[SB_RESTART_MAXOPT];
  double params[SB_RESTART_MAXOPT];
  double run_xoffb, run_xofft;           /* offsets of the state mapped on p */
  int ymap, ncopy, xskip;                /* y mapping, stack count, kx stride */
} sb_restart_info;
#define SB_RESTART_KEEP_VOR 1
int sb_write_restart(const char *path, const sb_params *p, const double *vor, const double *phi,
                     const double *u00, const double *w00, double time, double xoffb,
                     double xofft, double deltat);
int sb_read_restart(const char *path, const sb_params *p, double *vor, double *phi, double *u00,
                    double *w00, sb_restart_info *info);
int sb_read_restart_ex(const char *path, const sb_params *p, int flags, double *vor, double *phi,
                       double *u00, double *w00, sb_restart_info *info);

/* CUDA stream of the handle (cudaStream_t) and a blocking wait on it. */
void *sb_get_stream(sb_handle *h);
int sb_sync(sb_handle *h);

/* Sizes for a parameter set: out[0..7] = mx, mz, nkx(=mx/2), my, nz, mgalx,
 * mgalz, complex entries per box (= nkx*mz*my).  Host only. */
int sb_sizes(const sb_params *p, int *out);

/* The twiddle table of the length-n transforms as the device receives it:
 * factored = 0: e^{-2 pi i t/n}, t = 0..n-1, re/im interleaved (2n doubles;
 * the FP32 storage form); factored = 1: the FP64 form, 4n doubles per entry t
 * {mx, my, tau, swap} with e^{-2 pi i t/n} = (-i)^q c (1 + i tau), q the
 * nearest quarter turn, mx = (q < 2 ? c : -c), my = (odd q ? -mx : mx) and
 * swap = q & 1 as integer bits.  Host only (inspection and tests). */
int sb_fft_twiddles(int n, int factored, double *out);

/* Seeded divergence-free initial field (host only): random-phase modes with
 * E(k) ~ k^4 exp(-2 (k/k0)^2), rms velocity urms, written in the pencil layout.
 * A synthetic stand-in for the reference's getini (initcr.f90:664-822). */
int sb_seed_state(const sb_params *p, unsigned long long seed, double k0, double urms,
                  double *vor, double *phi, double *u00, double *w00);

/* Compact-scheme coefficients pr1, rh1*dy, pr2, rh2*dy^2 (7 each, index d+3)
 * as computed by prederiv1/prederiv2 (diffy_shear_hepta.f90:68-296). Host only. */
int sb_compact_coeffs(double *pr1, double *rh1h, double *pr2, double *rh2h);

const char *sb_last_error(void);
int sb_version(void);

#ifdef __cplusplus
}
#endif
#endif
