// defl.h -- deflation of the rigid-body modes of stiff passive inclusions, around
// the multigrid V-cycle.
//
// A stiff passive region (elements held at density 1) whose surroundings turn
// near-void during the optimisation moves almost freely: its six rigid-body
// motions are near-null modes of K (eigenvalues ~E_min), and a coarse grid whose
// elements are wider than the region does not represent them, so a multigrid
// preconditioned CG stalls.  The remedy is the deflation space Z of those motions
// (rigid-body-mode deflation of stiff inclusions, Jonsthovel, van Gijzen, Vuik and
// Scarpas, SIAM J. Sci. Comput. 35 (2013)), used here in the balancing (BNN) form
// that keeps the preconditioner symmetric positive definite:
//
//   z = P^T M P r + Q r,   Q = Z E^-1 Z^T,   E = Z^T K Z,   P = I - K Q,
//
// M the V-cycle.  Components: the passive solid elements, merged while two of
// them lie within 3 elements of each other, so that the node supports of K Z
// (the component's nodes and one ring around them) of different components are
// disjoint and E is block diagonal (6 x 6 per component).  Z, K Z and E live on
// those supports only; one application costs two dot-product launches, two 6 x 6
// block solves and three passes over the supports besides the V-cycle.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "am_common.cuh"
#include "kernels.cuh"
#include "defl_space.h"
#include "mg.h"

namespace amk {

struct Defl;

// Components of the elements flagged in solid (host, nel entries, element order of
// the device layout).  nullptr with *err = cudaSuccess when there is none, when
// they are more than a quarter of the elements or form more than
// DEFL_MAX_COMPONENTS components; *err set on an allocation failure.
Defl *defl_create(const Layout &L, const uint8_t *solid, cudaError_t *err);
void defl_destroy(Defl *d);
int defl_components(const Defl *d);

// For the operator (s64, M64 on plan64) and constraint bits mask (device, per
// node): Z masked to the free DOFs, K Z by six FP64 K*u of the fine grid (scratch
// vectors v, w of 3 L.cs doubles), E and its block inverse.  A block that is not
// positive definite (a component with no free DOF) is left out: its inverse is
// zero.  Synchronises the stream.
cudaError_t defl_setup(Defl *d, const KuLaunch &plan64, const Modal<double> &M64, const double *s64,
                       const uint8_t *mask, double *v, double *w, cudaStream_t st);

// z = P^T M P r + Q r with M = mg_apply(mg, .).  P r is formed in r itself on the
// supports (the V-cycle reads it there) and r is restored exactly afterwards.
cudaError_t defl_apply(Defl *d, Mg *mg, double *r, double *z, cudaStream_t st);

}  // namespace amk
