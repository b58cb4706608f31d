// kernels.cuh -- host-visible launchers of the GB300 SIMP engine kernels.
// Every launcher enqueues on `st` and returns the launch error (no host sync).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "am_common.cuh"

namespace amk {

// kernel launches issued so far (graph replays add their kernel-node count)
long long launch_count();
void count_launches(long long n);
// detail message returned by am_last_error() on this thread
void set_last_error(const char *msg);

// ---- tiled K*u (ku.cuh: FP64 / generic, ku2.cuh: FP32 warp-row form) --------
// Slack (entries) on both sides of a vector read by the unpredicated warp-row
// PCG kernel: the tiles' halo reaches one plane below node 0 and up to one plane,
// 2W+1 rows and 32 columns past the last plane of the last component.
inline long long ku2_slack(const Layout &L) { return (2 * L.sxy + 64LL * L.sx + 256 + 63) / 64 * 64; }

struct KuLaunch {
    int tx, ty;  // owned node columns per tile (one of the compiled shapes)
    int tz;      // node planes per tile
    int tiles_x, tiles_y, tiles_z;
    int warps;   // > 0: FP32 warp-row kernel (ku2.cuh) with this many warps
    int ntiles() const { return tiles_x * tiles_y * tiles_z; }
};
// fp64: ku.cuh shape for FP64; otherwise the FP32 warp-row kernel.  tz_hint <= 0
// picks the z chunking from a wave-quantisation cost model (resident CTAs per SM
// `ctas_per_sm`, `sms` multiprocessors).
KuLaunch ku_plan(const Layout &L, bool fp64, int tz_hint, int sms = 152);
// tiles of tx owned node columns x ty owned node rows, z chunking as above
KuLaunch ku_plan_shape(const Layout &L, int tx, int ty, int warps, int ctas_per_sm, int tz_hint, int sms = 152);

// ---- TMA-staged FP32 PCG K*u (ku3.cuh) -----------------------------------------
struct Ku3Maps;
// tensor maps of the problem's FP32 PCG vectors for tiles of `warps` (7 or 8)
// warps; the two padded arrays are ku3_padded_sizes() long and filled by
// ku3_pad().  Returns nullptr and sets *err on failure.  Free with ku3_free_maps.
Ku3Maps *ku3_make_maps(const Layout &L, const float *r, const float *pa, const float *pb, const float *dinv,
                       const uint8_t *mask_pad, const float *scale_pad, float *q, int warps, cudaError_t *err);
void ku3_free_maps(Ku3Maps *m);
// entries of the padded element-scale copy (rows of round_up(nx, 4)) and bytes of
// the padded constraint-bit copy (rows of round_up(nx+1, 16))
void ku3_padded_sizes(const Layout &L, long long *scale_entries, long long *mask_bytes);
// fills the padded copies from the element scales s32 (internal layout) and the
// per-node constraint bits
cudaError_t ku3_pad(const Layout &L, const float *s32, const uint8_t *mask, float *scale_pad, uint8_t *mask_pad,
                    cudaStream_t st);
// the launch plan: tiles of 28 node columns and 2 warps - 1 node rows (warps 8 or
// 7; 0 picks the one whose one-wave plan fills more CTA slots), two CTAs per SM
KuLaunch ku3_plan(const Layout &L, int warps = 0, int sms = 152);
// p = dinv r + beta p_prev, q = mask(K p), p.q -> S->alpha (ku_pcg's contract) with
// `stages` (3 or 4) shared-memory stages
cudaError_t ku3_pcg(const Ku3Maps *T, const KuLaunch &K, const Layout &L, const Modal<float> &M, double *partial,
                    Scalars *S, int stages, cudaStream_t st);
// The same step without a CTA barrier per plane (ku3b_kernel): p and q bitwise
// those of ku3_pcg; q and the new p are written to the raw vectors q and pa / pb
// (the map pair's parity as in ku3_pcg).  stages 4 or 5.
cudaError_t ku3b_pcg(const Ku3Maps *T, const KuLaunch &K, const Layout &L, const Modal<float> &M, float *q, float *pa,
                     float *pb, double *partial, Scalars *S, int stages, cudaStream_t st);
// the previous register-direct kernel (ku2_kernel) for the same PCG step (measurement)
cudaError_t ku2_pcg(const KuLaunch &K, const Layout &L, const Modal<float> &M, const float *s, float *pa, float *pb,
                    const float *r, const float *dinv, const uint8_t *mask, float *q, double *partial, Scalars *S,
                    cudaStream_t st);

template <typename T>
cudaError_t ku_plain(const KuLaunch &K, const Layout &L, const Modal<T> &M, const T *s, const T *u,
                     T *y, cudaStream_t st);
// p = dinv r + beta p_prev, q = mask(K p), partial p.q -> S->alpha.  p_prev / p are
// the ping-pong pair (pa, pb) chosen by the parity of S->it.  FP32 on the warp-row
// plan: pa, pb, r and dinv are read without bounds predicates and need
// ku2_slack(L) finite (zeroed) entries before and after their allocation.
template <typename T>
cudaError_t ku_pcg(const KuLaunch &K, const Layout &L, const Modal<T> &M, const T *s, T *pa, T *pb,
                   const T *r, const T *dinv, const uint8_t *mask, T *q, double *partial, Scalars *S,
                   cudaStream_t st);
// r = mask(f - K x) in FP64 with r.r, r.dinv.r -> S->res_rr / res_rz; optional ce.
cudaError_t ku_resid(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s,
                     const double *x, const double *f, const double *dinv, const uint8_t *mask,
                     double *r, double *ce, double *partial, Scalars *S, cudaStream_t st);
// The same residual with the element operator and node sums in double-float
// arithmetic on the FP32 pipes (kudf.cuh); FP64 inputs, outputs and sums.  The
// 32 x 4 FP64 tile plan only.
cudaError_t ku_resid_df(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s,
                        const double *x, const double *f, const double *dinv, const uint8_t *mask, double *r,
                        double *ce, double *partial, Scalars *S, cudaStream_t st);
// ku_dot (q = mask(K p), p.q -> the outer flexible CG's alpha) in double-float
cudaError_t ku_dot_df(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s, const double *p,
                      const uint8_t *mask, double *q, double *partial, Scalars *S, cudaStream_t st);

// ---- PCG vector kernels ------------------------------------------------------
// FP64 PCG: x += alpha p; r -= alpha q (p = the pair member written this
// iteration); rr, rz -> S (beta, stop tests: converged / reliable update due /
// max it).  Instantiated for double; the FP32 PCG uses pcg_update_df.
template <typename T>
cudaError_t pcg_update(const Layout &L, double *x, T *r, const T *pa, const T *pb, const T *q, const T *dinv,
                       double *partial, Scalars *S, int nblocks, cudaStream_t st);
// The same update with the iterate held as a double-float pair xh + xl (FP32
// vectors), the streams staged by bulk copies; one wave of 2 CTAs per SM (after
// ku_init_attributes).  A bulk-copy wait that runs out ends the solve with
// status ST_TIMEOUT.
// The iterate is folded every second iteration (even iterations owe alpha p to
// x in S->alpha_prev); pcg_df_settle pays an owed term once a solve stopped.
cudaError_t pcg_update_df(const Layout &L, float *xh, float *xl, float *r, const float *pa, const float *pb,
                          const float *q, const float *dinv, double *partial, Scalars *S, cudaStream_t st);
// x += S->alpha_prev p (p the last iteration's ping-pong member) if S->it is odd,
// then S->alpha_prev = 0; n = 3 cs entries
cudaError_t pcg_df_settle(long long n, float *xh, float *xl, const float *pa, const float *pb, Scalars *S,
                          int nblocks, cudaStream_t st);
int pcg_update_df_grid();
// reads `bytes` (a multiple of 16) of buf through L2 (measurement: cleans the
// L2 lines a flush write left dirty)
cudaError_t l2_flush_read(const void *buf, size_t bytes, cudaStream_t st);
// x = xh + xl, and (xh, xl) = the double-float split of x (n entries)
cudaError_t df_compose(const float *xh, const float *xl, double *x, long long n, int nblocks, cudaStream_t st);
cudaError_t df_split(const double *x, float *xh, float *xl, long long n, int nblocks, cudaStream_t st);
// x += xh + xl (n entries)
cudaError_t df_accumulate(const float *xh, const float *xl, double *x, long long n, int nblocks, cudaStream_t st);
// (re)start from the residual r (already masked); see pcg_start_kernel
template <typename T>
cudaError_t pcg_start(const Layout &L, const T *r, const T *dinv, double thr, double upd_factor, int maxit,
                      int restart, double *partial, Scalars *S, int nblocks, cudaStream_t st);
// r32 = r64 and, if x != nullptr, x = 0 (the FP32 sequence starts from the
// recomputed FP64 residual)
cudaError_t dc_inner_init(const Layout &L, const double *r64, float *r32, double *x,
                          const Scalars *S, int nblocks, cudaStream_t st);
// b = (float)a, n entries
cudaError_t to_float(const double *a, float *b, long long n, int nblocks, cudaStream_t st);
// r32 = mask(r64 - q32) (inner residual of an initial guess x with K x = q32)
cudaError_t inner_resid(const Layout &L, const double *r64, const float *q32, const uint8_t *mask, float *r32,
                        int nblocks, cudaStream_t st);
// x = 0 on every component whose bit is set in the per-node mask (a warm start
// keeps no value on constrained or orphan DOFs: the reference solution is 0 there)
cudaError_t zero_masked(const Layout &L, const uint8_t *mask, double *x, int nblocks, cudaStream_t st);
// outer flexible CG (FP64) with an inner preconditioner output z (FP64):
// z.r, z.q -> beta (first: 0) ; p = z + beta p ; q = mask(K p), p.q -> alpha ;
// x += alpha p, r -= alpha q, r.r
cudaError_t fcg_dots(const Layout &L, const double *z, const double *r, const double *q, int first,
                     double *partial, Scalars *S, int nblocks, cudaStream_t st);
cudaError_t fcg_direction(const Layout &L, const double *z, double *p, const Scalars *S, int nblocks,
                          cudaStream_t st);
cudaError_t ku_dot(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s, const double *p,
                   const uint8_t *mask, double *q, double *partial, Scalars *S, cudaStream_t st);
// the same q = mask(K p), p.q -> S->o_pq / o_alpha with the product in FP32
// (p rounded into p32, K p into q32, q and the dot in FP64)
cudaError_t ku_dot_f32(const KuLaunch &K32, const Layout &L, const Modal<float> &M, const float *s32, const double *p,
                       const uint8_t *mask, float *p32, float *q32, double *q, double *partial, Scalars *S,
                       int nblocks, cudaStream_t st);
cudaError_t fcg_update(const Layout &L, double *x, double *r, const double *p, const double *q, double *partial,
                       Scalars *S, int nblocks, cudaStream_t st);

// ---- set-up kernels ------------------------------------------------------------
// element scales from a device density (internal layout).  variant 0 (CPP):
// grid -1 or rho < rho_min -> 0, grid 1 -> 1, else emin + rho^p (1 - emin);
// variant 1 (PY): grid -1 -> 0, grid 1 -> 1, else (emin + rho^p (E - emin))/E.
cudaError_t scales(const Layout &L, const double *rho, const int8_t *grid, int variant, double p,
                   double emin, double rho_min, double E, double *s64, float *s32, cudaStream_t st, int d1 = 0);
// per-node inverse diagonal (KE[0][0] * sum of the adjacent scales), orphan DOFs
// (|diag| < 1e-15) joined to the constrained bits of `fixed_bits`.
cudaError_t diag_mask(const Layout &L, const double *s64, double d0, const uint8_t *fixed_bits,
                      double *dinv64, float *dinv32, uint8_t *mask, cudaStream_t st);

// ---- layout conversions --------------------------------------------------------
// reference DOF order <-> device component planes
cudaError_t dof_to_dev(const Layout &L, const double *src, double *dst, cudaStream_t st);
cudaError_t dev_to_dof(const Layout &L, const double *src, double *dst, cudaStream_t st);
template <typename T>
cudaError_t dof_to_dev_t(const Layout &L, const double *src, T *dst, cudaStream_t st);
template <typename T>
cudaError_t dev_to_dof_t(const Layout &L, const T *src, double *dst, cudaStream_t st);
// element array in host layout (0 z-fastest, 1 x-fastest) <-> internal x-fastest
template <typename T>
cudaError_t elem_to_dev(const Layout &L, const T *src, T *dst, int layout, cudaStream_t st);
template <typename T>
cudaError_t elem_from_dev(const Layout &L, const T *src, T *dst, int layout, cudaStream_t st);

// ---- filters ---------------------------------------------------------------------
struct Taps {
    const int4 *d;       // (dx, dy, dz, 0)
    const double *w;     // weight
    int n;
    int R;               // ceil(rmin): the halo of the shared-memory stencil (FP64, R <= 3)
};
// CPP: out = sum w rho_n x_n / sum w rho_n (neighbours in the grid), x if den <= 1e-15
template <typename T>
cudaError_t filter_cpp(const Layout &L, const Taps &tp, const double *x, const double *rho,
                       double *out, cudaStream_t st);
// PY: out = sum w x_n[reflect] ; mode 0 plain, 1 clip(out, lo, 1), 2 x := x*rho and
// out /= max(rho, 1e-3)
template <typename T>
cudaError_t filter_py(const Layout &L, const Taps &tp, const double *x, const double *rho,
                      double *out, int mode, double lo, cudaStream_t st);

// ---- sensitivities -----------------------------------------------------------------
// dc = -p rho^(p-1) ce over all elements (CPP) or design elements (PY, accumulated
// into dc with NaN -> 0); energy = sum s ce over non-void elements -> S->comp_energy
// (accumulate = 1 adds to S->comp_energy); fu = sum F.u over the listed DOFs.
cudaError_t sensitivities(const Layout &L, const double *rho, const double *ce, const double *s,
                          const uint8_t *design, int variant, double p, double *dc, int accumulate,
                          double *partial, Scalars *S, cudaStream_t st);
cudaError_t sparse_dot(const long long *idx, const double *val, int n, const double *u,
                       double *out, cudaStream_t st);
// sum of val^2 over the listed entries whose DOF is not masked (||F||^2 on the free DOFs)
cudaError_t masked_sqnorm(const long long *idx, const double *val, int n, long long cs,
                          const uint8_t *mask, double *out, cudaStream_t st);
// sets the shared-memory attributes of every compiled K*u kernel (call once,
// outside stream capture)
cudaError_t ku_init_attributes();
cudaError_t ku3_init_attributes();

// ---- OC ------------------------------------------------------------------------------
// Per-element terms of the OC update: a = rho sqrt(-dc), lo = rho - move,
// hi = rho + move, in FP64 (fp64 mode) or as double-float pairs (mixed).
struct OcBuffers {
    long long nel;
    double *a64, *lo64, *hi64;
    float2 *a32, *lo32, *hi32;
};
// computes the terms and resets the bisection state (l1, l2, t, pass, done)
cudaError_t oc_prepare(const OcBuffers &B, const double *rho, const double *dc, double move, int fp64,
                       int variant, Scalars *S, cudaStream_t st);
// one bisection pass: design volume at the current multiplier -> l1 / l2, stop test
cudaError_t oc_pass(const OcBuffers &B, const uint8_t *design, int fp64, int variant, double rho_min, double vf,
                    double n_design, double *partial, Scalars *S, int nblocks, cudaStream_t st);
// new density (FP64, from rho and dc) with the last pass's multiplier, max |change|,
// design-mask mean -> S
cudaError_t oc_final(const OcBuffers &B, const uint8_t *design, int fp64, int variant, double rho_min,
                     const double *rho, const double *dc, double move, double *rho_new, double *partial, Scalars *S,
                     int nblocks, cudaStream_t st);

}  // namespace amk
