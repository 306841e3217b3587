// kernels.cuh -- kernel declarations shared by the host orchestration.
#pragma once
#include <cuda_fp16.h>

#include <vector>

#include "common.cuh"
#include "vfs_poisson.h"

namespace vfs {

// Device pointers of the FormMetrics outputs (DA layout).
struct MetricPtrs {
  double *cent, *csi, *eta, *zet, *aj;
  double *icsi, *ieta, *izet, *iaj;
  double *jcsi, *jeta, *jzet, *jaj;
  double *kcsi, *keta, *kzet, *kaj;
  // the operator's nine face coefficients per DA point (g11 g21 g31 at i
  // faces, g12 g22 g32 at j faces, g13 g23 g33 at k faces), formed once per
  // grid by k_face_coef; null: formed in the assembly
  double *gface;
};

// setup.cu (compiled without FMA contraction)
__global__ void k_metrics_cell(Grid g, const double *coor, MetricPtrs m);
__global__ void k_face_coef(Grid g, MetricPtrs m, double *gface);
__global__ void k_metrics_mirror(Grid g, MetricPtrs m, int dir);
__global__ void k_metrics_periodic(Grid g, MetricPtrs m, int faces);
__global__ void k_metrics_face(Grid g, MetricPtrs m, int dir);
__global__ void k_count_dofs(Grid g, Box b, const double *nvert, int *block_count);
__global__ void k_scan_blocks(int *block_count, int nblocks, int *total);
__global__ void k_number_dofs(Grid g, Box b, const double *nvert, const int *block_off, int *gid_box);
__global__ void k_gid_da(Grid g, Box b, const int *gid_box, int *gid_da);
__global__ void k_rhs2(Grid g, Box b, const double *nvert, const uint8_t *rowtype, const double *ucont,
                       const double *aj, double dt, double st, double coeff, int poisson, double *rhs, double *partial);
__global__ void k_rhs2_shift(Grid g, Box b, const double *nvert, const double *aj, const double *sums, int poisson,
                             double *rhs);
__global__ void k_vflux_sum(Grid g, const double *nvert, MetricPtrs m, double *ucont, int flg, int pass,
                            double *partial);
__global__ void k_vflux_apply(Grid g, const double *nvert, MetricPtrs m, double *ucont, int flg, double corr);
__global__ void k_vflux0_sum(Grid g, const double *nvert, MetricPtrs m, double *ucont, double *partial);
__global__ void k_vflux0_apply(Grid g, const double *nvert, MetricPtrs m, double *ucont, double corr, int zero);
__global__ void k_periodic_cmpnts(Grid g, const double *src, double *dst);
__global__ void k_contra2cart(Grid g, const double *nvert, MetricPtrs m, const double *lu, double *ucat);
__global__ void k_zero_solid(Grid g, const double *nvert, double *ucat);
__global__ void k_cellfield_restrict(Grid gh, Grid gc, int cx, int cy, int cz, const double *fh, double *fc);
__global__ void k_assemble(Grid g, Box b, const double *nvert, MetricPtrs m, int scale, int filter, int split, double *A,
                           uint8_t *rowtype, LevelSet ls);
__global__ void k_assemble_fine(Grid g, Box b, const double *nvert, MetricPtrs m, double *A0, uint8_t *rowtype0,
                                double *A1, uint8_t *rowtype1, LevelSet ls);
__global__ void k_assemble_rows(Grid g, Box b, const double *nvert, MetricPtrs m, int scale, int filter, int split,
                                double *A, uint8_t *rowtype, LevelSet ls, const int *rows, const int *nrows);
__global__ void k_assemble_fine_rows(Grid g, Box b, const double *nvert, MetricPtrs m, double *A0, uint8_t *rowtype0,
                                     double *A1, uint8_t *rowtype1, LevelSet ls, const int *rows, const int *nrows);
__global__ void k_mask_changed(size_t N, const double *a, const double *b, uint8_t *chg);
__global__ void k_dilate_axis(Grid g, int axis, int R, const uint8_t *src, uint8_t *dst);
__global__ void k_list_rows(Grid g, Box b, const uint8_t *flag, int *rows, int *nrows, uint8_t *colflag);
__global__ void k_projection_coef(Grid g, Box b, MetricPtrs m, double *pc);
__global__ void k_level_masks(Grid g, Box b, const double *nvert, uint8_t *blank, double *w64, float *w32,
                              double *aj_box, const double *aj_da);
__global__ void k_rhs(Grid g, Box b, const double *nvert, const double *ucont, const double *aj, double dt,
                      double st, double coeff, double *rhs, double *partial);
__global__ void k_reduce_rows(const double *partial, int nb, int nrow, double *out);
__global__ void k_rhs_nullspace(Grid g, Box b, const double *nvert, const double *aj, const double *sums,
                                double *rhs);
__global__ void k_fully_blocked(Grid g, const double *nvert, int *ksk, int *unblocked);
__global__ void k_nullspace_sums(Grid g, const double *nvert, const int *ksk, int multi, const double *x,
                                 double *partial);
__global__ void k_nullspace_apply(Grid g, const double *nvert, const int *ksk, int multi, double shift0,
                                  double shift1, double *x);
__global__ void k_mean_partial(Box b, const uint8_t *fluid, const double *x, double *partial);
__global__ void k_fluid_mask(Grid g, Box b, const double *nvert, uint8_t *fluid);
__global__ void k_mean_shift(double *sums);
__global__ void k_box_to_da_phi(Grid g, Box b, const double *nvert, const double *x, double *phi,
                                const double *shift);
__global__ void k_da_to_box(Grid g, Box b, const double *da, double *x);
__global__ void k_box_to_da(Grid g, Box b, const double *x, double *da);
__global__ void k_update_pressure(Grid g, const double *nvert, const double *phi, double *p);
__global__ void k_periodic_copy2(Grid g, double *p, double *phi);
__global__ void k_projection(Grid g, Box b, const double *nvert, const double *phi, const double *pc, double dt,
                             double st, double coeff, double *ucont, MetricPtrs m, LevelSet ls);
__global__ void k_periodic_faces(Grid g, double *ucont);
__global__ void k_divergence(Grid g, Box b, const double *nvert, const double *ucont, const double *aj,
                             double *partial);
__global__ void k_reduce_max(const double *partial, int nb, double *out);
__global__ void k_coarse_nodes(Grid gf, Grid gc, int cx, int cy, int cz, const double *cf, double *cc);
__global__ void k_nvert_restrict(Grid gh, Grid gc, int cx, int cy, int cz, const double *nh, double *nc);
__global__ void k_nvert_fill(Grid gc, const double *src, double *dst);
__global__ void k_restrict_f32(Box bf, Box bc, int cx, int cy, int cz, const float *rf, const float *wf,
                               const uint8_t *blank_c, float *out);
__global__ void k_restrict_f64(Box bf, Box bc, int cx, int cy, int cz, const double *rf, const double *wf,
                               const uint8_t *blank_c, double *out);
__global__ void k_prolong_f32(Box bf, Box bc, int cx, int cy, int cz, const float *xc, const uint8_t *blank_c,
                              const uint8_t *blank_f, float *xf, int add);
__global__ void k_prolong_f32_split(Box bf, Box bc, int cx, int cy, int cz, const float *xc, const uint8_t *blank_c,
                              const uint8_t *blank_f, float *xf, int add);
__global__ void k_prolong_f64(Box bf, Box bc, int cx, int cy, int cz, const double *xc, const uint8_t *blank_c,
                              const uint8_t *blank_f, double *xf, int add);

// solve.cu (hot loop kernels)
#define TYPED_DECL(T, S)                                                                                 \
  __global__ void k_residual_##S(Box b, const T *A, const T *x, const T *rhs, T *r, int color);          \
  __global__ void k_line_lu_##S(Box b, const double *A64, T *inv, T *cp, const uint8_t *colflag);        \
  __global__ void k_line_sweep_##S(Box b, const T *A, const T *inv, const T *cp, const T *x, const T *rhs, \
                                   T *xo, T omega, int zero_guess);                                      \
  __global__ void k_line_tri_##S(Box b, const T *r, const T *Asp, const T *inv, const T *cp, T *x, T omega,  \
                                 int zero_guess, int color);                                             \
  __global__ void k_coarsest_##S(int nd, const int *dmap, const int *didx, const double *dinv, const T *rhs, T *x, \
                                 int n);                                                                     \
  __global__ void k_cast_planes_##S(const double *src, T *dst, size_t n);
TYPED_DECL(float, f32)
TYPED_DECL(double, f64)
#undef TYPED_DECL

__global__ void k_pack16(size_t n, const double *A, __half2 *C, float *D);
__global__ void k_pack16_rows(Box b, const double *A, __half2 *C, float *D, float *A32, const int *rows,
                              const int *nrows);
__global__ void k_residual16(Box b, const __half2 *C, const float *D, const float *x, const float *rhs, float *r,
                             int color);
__global__ void k_residual16_split(Box b, const __half2 *C, const float *D, const float *x, const float *rhs, float *r,
                             int color);
__global__ void k_line_tri_f32_split(Box b, const float *r, const float *Asp, const float *inv, const float *cp, float *x,
                                     float omega, int zg, int color);
// Checkerboard zebra colour with the residual formed in the line kernel:
// _oz counts the launch's colour as zero (its loads are masked), _z every x
// (r = rhs).
#define LINE_FUSED_DECL(NAME)                                                                                   \
  __global__ void NAME(Box b, const __half2 *C, const float *D, const float *xo, const float *xn, const float *rhs, \
                       const float *Asp, const float *inv, const float *cp, float *xd, float omega, int color);
LINE_FUSED_DECL(k_line_fused16)
LINE_FUSED_DECL(k_line_fused16_oz)
LINE_FUSED_DECL(k_line_fused16_z)
#undef LINE_FUSED_DECL
__global__ void k_apply64(Box b, const double *A, const double *x, double *y);
__global__ void k_residual64(Box b, const double *A, const double *x, const double *rhs, double *r, double *partial);
__global__ void k_residual64r(Box b, const double *A, const double *x, const double *rhs, double *r);
// Gram-Schmidt rows of the reduced values (solve.cu): Q.u at 0.., Q.w at
// kGsB.., u.u and u.w at kGsUU, r, h and 1/r at kGsR.
// kGsTile cells per thread in k_gs_dots* and k_gs_update (256-thread blocks).
constexpr int kGsB = 64, kGsUU = 128, kGsR = 130, kGsTile = 8;
#define GS_DOTS_DECL(NV)                                                                             \
  __global__ void k_gs_dots##NV(size_t n, int v0, const double *const *Q, const double *u, const double *w, \
                                int first, double *partial);
GS_DOTS_DECL(0)
GS_DOTS_DECL(1)
GS_DOTS_DECL(2)
GS_DOTS_DECL(3)
GS_DOTS_DECL(4)
GS_DOTS_DECL(5)
GS_DOTS_DECL(6)
GS_DOTS_DECL(7)
GS_DOTS_DECL(8)
#undef GS_DOTS_DECL
#define CGS_DOTS_DECL(NV) \
  __global__ void k_cgs_dots##NV(size_t n, int v0, const double *const *Q, const double *w, double *partial);
CGS_DOTS_DECL(1)
CGS_DOTS_DECL(2)
CGS_DOTS_DECL(3)
CGS_DOTS_DECL(4)
CGS_DOTS_DECL(5)
CGS_DOTS_DECL(6)
CGS_DOTS_DECL(7)
CGS_DOTS_DECL(8)
#undef CGS_DOTS_DECL
__global__ void k_cgs_reduce(const double *partial, int nb, const double *dsv, double *red);
__global__ void k_cgs_update(size_t n, int nv, const double *const *Q, const double *red, double *w,
                             double *partial);
__global__ void k_gs_reduce(const double *partial, int nb, int nv, double *red);
__global__ void k_gs_coef(int nv, double *red);
__global__ void k_gs_update(size_t n, int nv, const double *const *Q, const double *red, double *u, double *w,
                            double *partial);
__global__ void k_axpy_multi(size_t n, int nv, const double *const *Z, const double *coef, double *x);
__global__ void k_scale_to(size_t n, const double *v, double s, const double *sinv, const double *scale,
                           double *out);
__global__ void k_scale_to32(size_t n, const double *v, float s, const float *sinv, const float *scale, float *out,
                             int split_nx);
__global__ void k_reduce_norm(const double *partial, int nb, double *out, float *out32);
__global__ void k_to64(size_t n, const float *x32, const double *x64, double *out, int split_nx);
__global__ void k_sumsq(size_t n, const double *x, double *partial);
// history projection of the initial guess (at most kHistMax solutions:
// the newest and the differences of consecutive ones)
constexpr int kHistMax = 12;
struct HistPtrs {
  const double *p[kHistMax];
};
// v . Y_j (j < k) and v . v as block partials (row j, row k)
void launch_hist_dots(cudaStream_t st, int blocks, size_t n, const HistPtrs &Y, int k, const double *v,
                      double *partial);
// x = sum_j c_j X_j, r = b - sum_j c_j Y_j and the partials of ||r||^2
void launch_hist_combine(cudaStream_t st, int blocks, size_t n, const HistPtrs &X, const HistPtrs &Y, int k,
                         const double *c, const double *b, double *x, double *r, double *partial);
// a converged solve into the newest solution and a difference slot, with
// the new Gram entries as block partials (rows as in hist_push_body)
void launch_hist_push(cudaStream_t st, int blocks, size_t n, const double *x, const double *b, const double *r,
                      double *Xn, double *Yn, double *dX, double *dY, const HistPtrs &E, int m, bool first,
                      double *partial);
__global__ void k_fluid_moments(size_t n, const uint8_t *fluid, const double *z, double mean, int pass,
                                double *partial);

// Hand-off from a handle to the surface search (ibm.cu): its stream, grid,
// DA-layout cell centres and launch counter.
// One body's IB node records in device memory (built by the surface
// search in ibm.cu, applied by vfs_poisson_ibm_interpolate; the handle owns
// and frees them).
struct IbmBody {
  int n_nodes = 0, n_elmt = 0, n_v = 0;
  vfs_ibm_node *nodes = nullptr;
  int *tri = nullptr;
};
// device buffers of the surface search, kept by the handle and grown on
// demand (no allocation or free, and so no device synchronisation, per body)
struct IbmScratch {
  void *buf[11] = {};
  size_t cap[11] = {};
  // bounds of the cell centres over blocks of 8x8x8 interior cells (6
  // doubles each), formed by the first search after the grid was set
  double *bbox = nullptr;
  size_t bbox_cap = 0;
  bool bbox_valid = false;
  int *hits = nullptr;  // the blocks that meet a body's hash box
  size_t hits_cap = 0;
};
struct IbmContext {
  cudaStream_t stream;
  Grid g;
  const double *cent;
  int64_t *launches;
  std::vector<IbmBody> *bodies;
  IbmScratch *scratch;
};
// ibm.cu: the IB interpolation and IB_BC kernels (launched by poisson.cu)
__global__ void k_ibm_apply(Grid g, const vfs_ibm_node *nodes, int n_nodes, const int *tri, const double *u_surf,
                            const double *nvert, const double *lucat, const double *lp, double *ucat, double *p);
__global__ void k_ibm_faces(Grid g, const double *nvert, const double *lu, const double *icsi, const double *jeta,
                            const double *kzet, double f, int b0, int b1, int b2, int b3, int b4, int b5,
                            double *ucont);
__global__ void k_ib_bc_faces(Grid g, const double *nvert, const double *lu, const double *icsi,
                              const double *jeta, const double *kzet, int immersed, int b0, int b1, int b2, int b3,
                              double *ucont);
__global__ void k_ib_bc_edges(Grid g, const double *uold, int b0, int b1, int b2, int b3, int b4, int b5,
                              double *ucont);

}  // namespace vfs
