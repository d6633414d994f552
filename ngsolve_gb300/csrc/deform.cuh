// deform.cuh -- curved elements through a mesh deformation field (the
// reference's MeshAccess::SetDeformation, comp/meshaccess.cpp:1573-1580,
// applied by ALE_ElementTransformation, :240-340):
//   x(xi) = x_mesh(xi) + d(xi),   J(xi) = J_mesh(xi) + grad_xi d(xi),
// d a vector field in the H1 space of some order k on the same mesh (component-
// major DOFs, VectorH1 without interleaving).  Every geometry kernel adds the
// field's reference gradient at its point through deform_add; the element maps
// are then non-affine, so hexes take the per-point metric paths and tets the
// per-point B^T D B path.
#pragma once
#include "common.cuh"
#include "basis.cuh"

namespace gh1 {

struct DeformView {
  const double* d = nullptr;     // [3][ndof] component-major; nullptr: no deformation
  int64_t ndof = 0;
  int et = 8, k = 1, nloc = 0;
  const int32_t* eldofs = nullptr;  // tet: element DOFs of the field's space, reference order
  const int32_t* tdof = nullptr;    // hex: signed tensor DOF table of the field's space
  int tstride = 0;
  const int32_t* el = nullptr;      // element vertex numbers (tet shape orientation)
};

// J[3r+c] += d x_r / d xi_c of the field, disp[r] += d_r (disp may be null)
__device__ inline void deform_add(const DeformView& dv, int e, double x, double y, double z, double* J, double* disp) {
  if (!dv.d) return;
  if (dv.et == 8) {
    const int N = dv.k + 1;
    Dual3 px[MAX_HEX_ORDER + 1], py[MAX_HEX_ORDER + 1], pz[MAX_HEX_ORDER + 1];
    hex_psi<Dual3>(dv.k, Dual3(x, 1, 0, 0), px);
    hex_psi<Dual3>(dv.k, Dual3(y, 1, 0, 0), py);
    hex_psi<Dual3>(dv.k, Dual3(z, 1, 0, 0), pz);
    const int32_t* T = dv.tdof + (size_t)e * dv.tstride;
    for (int a = 0; a < N; a++)
      for (int b = 0; b < N; b++)
        for (int c = 0; c < N; c++) {
          const int t = T[(a * N + b) * N + c];
          const double s = t < 0 ? -1.0 : 1.0;
          const int64_t dof = t & 0x7fffffff;
          const double g[3] = {s * px[a].dx * py[b].v * pz[c].v, s * px[a].v * py[b].dx * pz[c].v,
                               s * px[a].v * py[b].v * pz[c].dx};
          for (int r = 0; r < 3; r++) {
            const double dr = dv.d[r * dv.ndof + dof];
            J[3 * r] += dr * g[0];
            J[3 * r + 1] += dr * g[1];
            J[3 * r + 2] += dr * g[2];
            if (disp) disp[r] += dr * s * px[a].v * py[b].v * pz[c].v;
          }
        }
  } else {
    constexpr int MAXL = (MAX_TET_ORDER + 1) * (MAX_TET_ORDER + 2) * (MAX_TET_ORDER + 3) / 6;
    Dual3 sh[MAXL];
    const int vn[4] = {dv.el[(size_t)e * 4], dv.el[(size_t)e * 4 + 1], dv.el[(size_t)e * 4 + 2], dv.el[(size_t)e * 4 + 3]};
    tet_shapes<Dual3>(dv.k, vn, Dual3(x, 1, 0, 0), Dual3(y, 0, 1, 0), Dual3(z, 0, 0, 1), sh);
    const int32_t* D = dv.eldofs + (size_t)e * dv.nloc;
    for (int i = 0; i < dv.nloc; i++) {
      const int64_t dof = D[i];
      for (int r = 0; r < 3; r++) {
        const double dr = dv.d[r * dv.ndof + dof];
        J[3 * r] += dr * sh[i].dx;
        J[3 * r + 1] += dr * sh[i].dy;
        J[3 * r + 2] += dr * sh[i].dz;
        if (disp) disp[r] += dr * sh[i].v;
      }
    }
  }
}

// the deformation view of a mesh (empty without a deformation)
inline DeformView deform_view(const gh1_mesh* m) {
  DeformView dv;
  const gh1_space* s = m->def_space;
  if (!s || !m->d_def.p) return dv;
  dv.d = m->d_def.p;
  dv.ndof = s->ndof;
  dv.et = s->et;
  dv.k = s->p;
  dv.nloc = s->nloc;
  dv.eldofs = s->d_eldofs.p;
  dv.tdof = s->d_tdof.p;
  dv.tstride = s->tstride;
  dv.el = m->d_el.p;
  return dv;
}

}  // namespace gh1
