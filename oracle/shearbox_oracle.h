/*
 * shearbox_oracle.h -- CPU FP64 restatement of the shearing-box RK3 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle exists so that tests/, the smoke check
 * and the CPU-baseline leg of bench.py can check the CUDA library against the
 * reference algorithm.  The product (shear_nnf_gb300/) never links, imports or
 * calls it.
 *
 * Parity status: the reference (Fortran + FFTW + MPI) cannot be compiled in this
 * environment and ships no golden vectors, so the oracle is pinned against the
 * reference's own analytic checks instead: the rapid-distortion (RDT) solution
 * rdtfunc (operators.f90:1516-1562, the check recorded in log_changes for
 * rev.428-430), the design conditions of the compact schemes (prederiv1/2), and
 * numpy's DFT for the x/z transforms.  It is not pinned to reference binary
 * outputs.
 *
 * Layouts follow the reference exactly:
 *   pencil   vor(0:2*my-1, 0:mx1, 0:mz1)  real, i.e. complex(0:my1,0:mx1,0:mz1),
 *            y fastest (cross.f90:32-33);
 *   plane    complex(0:mx1, 0:mz1, 0:my1), kx fastest (cross.f90:1144).
 */
#ifndef SHEARBOX_ORACLE_H
#define SHEARBOX_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  int mgalx, my, mgalz;   /* physical grid (hre2.dat record 1) */
  double Re, alp, Ly, gam, s, chi, CFL; /* hre2.dat record 2 (Ly read directly) */
  double vbulk;           /* u2c(0,0) override in hvhg (cross.f90:1276) */
  double fixed_dt;        /* >0: fixed time step (ifix_dt branch, cross.f90:1608) */
  int readflag;           /* 0: initial umax from s/uprim on the first step (cross.f90:1208) */
  double uprim;           /* hre2.dat record 4 */
  int nhist;              /* statistics every nhist steps (cross.f90:344) */
  double etime, dumptime, dtimag; /* end/dump times (cross.f90:1694-1711) */
  int keep_laminar;       /* 1: no stop on laminarisation (cross.f90:2106-2115) */
  int les;                /* iuse_LES: Smagorinsky model (cross.f90:1291-1406) */
  int les_visc;           /* iadd_visc: molecular viscosity kept with the model */
  double cs;              /* Cles, the Smagorinsky constant (initcr.f90:1964,2148) */
  int ydeal;              /* iydealiasing: 0 none, 1 y 2/3 rule on kx=0 and the mean modes,
                           * 2 the moving-frame variant on every kx (dealiasing_y,
                           * operators.f90:352-467), 3 compact y-filter
                           * (cross.f90:214-227,476-490) */
  int temperature;        /* itemperature: Boussinesq scalar tb of crosst (crosst.f90:3-1310) */
  double fkappa, bym, gbeta; /* its diffusivity, mean gradient and buoyancy factor
                           * (hre3.dat keyword itemperature, initcr.f90:1996-2011) */
  int damping;            /* iadd_damping: window damping of the mean forcing rf0u
                           * (add_damping, operators.f90:42-84; cross.f90:625-626) */
  double damp_up, damp_aa; /* its permeability and half width / Lz (initcr.f90:2128) */
  int force;              /* iadd_force: 1, 2 streamwise-roll force on hv(kx=0, kz=1)
                           * (add_force, operators.f90:1-40); -1 xforce on rf0u
                           * (cross.f90:610-624) */
  double force_roll, xforce; /* their amplitudes (initcr.f90:2103-2118) */
  int implicit_visc;      /* 1: viscous terms semi-implicit (explicit = 0,
                           * cross.f90:797-989, crosst.f90:916-1195,
                           * initcr.f90:1976-1984); not with LES
                           * (initcr.f90:2179), fkappa > 0 with the temperature */
} orc_params;

/* one .cfbin record per statistics step (cross.f90:2087):
 * time, Deltat, uner(1:10), CFL, CFLv, umax(1:3), xoffb, xofft, umax(0), uner2(1:4) */
#define ORC_TRACE_LEN 24
/* crosst writes the same record followed by tbmax, tner(1:4) (crosst.f90:2456-2458) */
#define ORC_TRACE_LEN_T 29

void *orc_create(const orc_params *p);
void orc_destroy(void *h);
/* out[0..7] = mx, mz, nkx(=mx/2), my, nz, mgalx, mgalz, buffsize(=mx*mz*my) */
void orc_sizes(void *h, int *out);
void orc_coeffs(void *h, double *pr1, double *rh1, double *pr2, double *rh2,
                double *dy);
void orc_set_threads(int n);

/* cross(): nstep RK3 steps in place on pencil-layout arrays.  trace receives up
 * to nstep records; *ntrace the count; *istop the stop flag; *deltat the last
 * Deltat.  Returns the number of completed steps. */
int orc_cross(void *h, double *vor, double *phi, double *u00, double *w00,
              double *time, double *xoffb, double *xofft, int nstep,
              double *trace, int *ntrace, int *istop, double *deltat);

/* crosst(): cross with the scalar tb (pencil layout like vor) and its mean
 * profile tb00(0:my1); needs temperature = 1.  Trace records have
 * ORC_TRACE_LEN_T doubles. */
int orc_crosst(void *h, double *vor, double *phi, double *u00, double *w00, double *tb,
               double *tb00, double *time, double *xoffb, double *xofft, int nstep,
               double *trace, int *ntrace, int *istop, double *deltat);

/* statistics accumulated over the last cross/crosst call (hist 'f', 'p', 'w',
 * cross.f90:1796-2121; crosst.f90:2201-2210,2364-2374): stats and stats2
 * (23 x my), spectra spec and spec2 (8 x nkx x mz), the temperature's tstats
 * (5 x my) and tspec (4 x nkx x mz), first index fastest; any pointer may be
 * NULL */
void orc_statistics(void *h, double *stats, double *stats2, double *spec, double *spec2,
                    double *tstats, double *tspec, int *nacum, double *total_dt);

/* building blocks, one y-line (complex: m=2, real: m=1) */
void orc_filterc(void *h, const double *u, double *du, double shp_re, double shp_im, int m);
/* rfty / cfty on one y-line (packed real line of my+2 doubles, or complex) */
void orc_rfty(void *h, double *u, int iopt);
void orc_cfty(void *h, double *u, int iopt);
/* physical fields of convh5 (u v w ox oy oz Q R Qs Rs Qw by mask bits 0..10),
 * each [my][mgalz][mgalx]; returns the number of fields written */
int orc_physical(void *h, const double *vor, const double *phi, const double *u00,
                 const double *w00, double xoffb, double xofft, unsigned mask, double *out);
/* dealiasing_y (iydealiasing 1, 2) on pencil-layout state arrays */
void orc_dealiasing_y(void *h, double *vor, double *phi, double *u00, double *w00, double fac);
void orc_derivyc(void *h, const double *u, double *du, double shp_re,
                 double shp_im, double shm_re, double shm_im, int iord, int m);
void orc_lapcdy(void *h, const double *u, double k2, double *p, double shp_re,
                double shp_im, double shm_re, double shm_im, int m);
/* one plane: iopt=+1 fou(complex 0:mx1,0:mz1) -> phys((mgalx+2) x mgalz);
 *            iopt=-1 phys -> fou */
void orc_fourxz(void *h, double *fou, double *phys, int iopt);
/* plain complex FFT of length n (sign -1 forward, +1 backward, unnormalised) */
void orc_fft(int n, double *data, int sign);
/* seeded divergence-free field of the benchmark configurations (E(k) ~ k^4
 * exp(-2 (k/k0)^2), rms urms), pencil layout; returns 0, or -1 without memory */
int orc_seed_state(int mgalx, int my, int mgalz, double alp, double gam, double Ly,
                   unsigned long long seed, double k0, double urms, double *vor, double *phi,
                   double *u00, double *w00);

#ifdef __cplusplus
}
#endif
#endif
