// sb_kernels.h -- launch entry points of the device kernels (internal).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "sb_common.cuh"

namespace sb {
int plane_cb(int mgalz);
int plane_t2_default(int mgalx);
bool plane3_fits(const Grid &g, int cb);
bool supported_grid(int mgalx, int mgalz);
cudaError_t launch_plane(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st);
int les_cb(int mgalz);
cudaError_t launch_les(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st);
cudaError_t launch_lineL(const Grid &g, const Bufs &bf, cudaStream_t st);
cudaError_t launch_filter(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t launch_ydeal(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t launch_meand1(const Grid &g, const Bufs &bf, cudaStream_t st);
cudaError_t launch_spectra(const Grid &g, const Bufs &bf, cudaStream_t st);
cudaError_t launch_physical(const Grid &g, const Bufs &bf, unsigned mask, double *out,
                            cudaStream_t st);
bool supported_ylen(int my);
cudaError_t launch_yop(int my, int nlines, double *c, long ldc, int iopt, int real, cudaStream_t st);
cudaError_t launch_filter_rhs(int nlines, int N, const double *u, long ldu, double *out, long ldo,
                              const double *shp, const double r[5], cudaStream_t st);
cudaError_t prepare_line(const Grid &g);
int line_segments();
bool line_segments_supported(int nseg);
size_t line_smem(const Grid &g);
cudaError_t launch_lineA(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t launch_lineB(const Grid &g, const Bufs &bf, int mode, cudaStream_t st);
// the substep's y-line work in one kernel (k_lineF) in place of k_lineA +
// k_lineB, where line_fused_ok(g)
cudaError_t launch_lineF(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
bool line_fused_ok(const Grid &g);
// the semi-implicit viscous branch: factor tables of the substep (k_hfac)
// and the y-line kernel (k_lineI)
cudaError_t launch_hfac(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t launch_lineI(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
bool line_implicit_ok(const Grid &g);
cudaError_t launch_setconj(const Grid &g, const Bufs &bf, cudaStream_t st);
cudaError_t launch_scalar(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t launch_tables(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t launch_finish(const Grid &g, const Bufs &bf, cudaStream_t st);
cudaError_t launch_pencil_to_plane(const Grid &g, const double *pen, double *dst, cudaStream_t st);
cudaError_t launch_plane_to_pencil(const Grid &g, const double *src, double *pen, cudaStream_t st);
cudaError_t fp64_peak(double *tflops, cudaStream_t st);
long op_threads(int nlines);
cudaError_t launch_op_line(int nlines, int N, const double *u, long ldu, double *out, long ldo,
                           double *ybuf, const Fac &F, const double *shp, const double *shm,
                           const double r[4], int anti, cudaStream_t st);
long packed_length(const Grid &g);
cudaError_t launch_pack(const Grid &g, const double *vor, const double *phi, const double *mu,
                        double *x, const double sca[3], double sx, double sz, cudaStream_t st);
cudaError_t launch_unpack(const Grid &g, const double *x, double *vor, double *phi, double *mu,
                          const double sca[3], cudaStream_t st);
cudaError_t launch_tangent(const Grid &g, const double *x, double *out, int dir,
                           cudaStream_t st);
int noalloc_derivyc(int my, double Ly, int iord, int nlines, const double *u, long ldu,
                    double *out, long ldo, const double *shp, const double *shm, void *stream,
                    std::string *err);
}  // namespace sb
