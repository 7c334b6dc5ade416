// General ghost-cell and grid-transfer utilities on a device forest, for codes
// other than the multigrid solver, and the VTK writer of leaf data:
//
//   a$D_prolong0/1/2_from          src/m_aX_prolong.f90:22-348
//   a$D_restrict_tree              src/m_aX_restrict.f90:21-64
//   a$D_gc_tree with sides_rb = a$D_gc_prolong0 / a$D_gc_interp /
//     a$D_gc_interp_lim / mg$D_sides_rb   src/m_aX_gc.f90:28-358, m_aX_mg.f90:262-350
//   a$D_gc2_box with a$D_gc2_prolong1 / a$D_bc2_neumann_zero
//                                  src/m_aX_gc.f90:420-634
//   a$D_consistent_fluxes          src/m_aX_core.f90:811-945
//   a$D_write_vtk                  src/m_aX_io.f90:115-310, src/m_vtk.f90
//
// They act on any cell variable of the forest (phi, rhs, tmp or the extra
// variables of afv_forest_add_vars) and on its face variables, one launch
// per level for every tree. These are not on the solver's hot path: each
// kernel takes one thread per output value, reads its inputs straight from
// global memory and keeps the reference's expression order, so that results
// are bit-identical to the reference's routines (the library is compiled with
// -fmad=false).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "afivo_gb300.h"
#include "forest.hpp"

namespace afv {

int forest_exchange_plan(Forest& F, std::string& err);

namespace xdev {

struct XT {
  const int* nb;            // [s*2D+f] neighbour slot, -1 refinement boundary, -2 physical
  const int* parent;        // [s]
  const int* first_child;   // [s]
  const int* lvl;           // [s]
  const int* qd;            // [s] child-number bits (levels >= 2), else -1
  const long long* offg;    // [s]
  const SlotDesc* desc;     // [s]
  const double* bcval;      // boundary values of the sampled sides_bc records
  const double* rmin;       // [s*D+d] lower corner of each box
  int cyl;                  // cylindrical trees (2-D)
};

// a2_cyl_child_weights (src/m_aX_t.f90:516-528): weights of the inner and
// outer child at cell index i of a box with lower radius r0 and cell size dr
// (the cell centre's radius, a2_cyl_radius_cc, :508-514).
__device__ __forceinline__ void cyl_weights(double r0, double dr, int i, double& inner, double& outer) {
  const double r = r0 + (i - 0.5) * dr;
  const double tmp = 0.25 * dr / r;
  inner = 1 - tmp;
  outer = 1 + tmp;
}

template <int D>
__device__ __forceinline__ long long gi(int ng, int i, int j, int k) {
  return (long long)i + (long long)ng * (j + (D == 3 ? (long long)ng * k : 0));
}

// Offset of a child's quadrant in its parent (a$D_get_child_offset,
// src/m_aX_t.f90:362-374): 0 on levels <= 1.
__device__ __forceinline__ int child_off(const XT& t, int c, int d, int hnc) {
  return t.lvl[c] > 1 ? ((t.qd[c] >> d) & 1) * hnc : 0;
}

// a$D_prolong{0,1,2}_from for every parent of a level: one thread per coarse
// cell of a child's quadrant, writing the 2^D fine cells it covers.
template <int D>
__global__ void k_prolong(XT t, const int* __restrict__ parents, int np, int nch, int ncp, int ncc,
                          const double* __restrict__ src, double* __restrict__ dst, int order, int add) {
  const int hnc = ncc / 2;
  const long long per_child = D == 2 ? (long long)hnc * hnc : (long long)hnc * hnc * hnc;
  const long long n = (long long)np * nch * per_child;
  const int ngp = ncp + 2, ngc = ncc + 2;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < n;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % per_child);
    const int ch = (int)((it / per_child) % nch);
    const int P = parents[it / per_child / nch];
    const int C = t.first_child[P] + ch;
    const int i = q % hnc + 1, j = (q / hnc) % hnc + 1, k = D == 3 ? q / (hnc * hnc) + 1 : 0;
    const int ic = i + child_off(t, C, 0, hnc), jc = j + child_off(t, C, 1, hnc);
    const int kc = D == 3 ? k + child_off(t, C, 2, hnc) : 0;
    const double* p = src + t.offg[P];
    double* c = dst + t.offg[C];
    const int i_f = 2 * i - 1, j_f = 2 * j - 1, k_f = D == 3 ? 2 * k - 1 : 0;
    auto P_ = [&](int a, int b, int e) { return p[gi<D>(ngp, a, b, e)]; };
    auto C_ = [&](int a, int b, int e) -> double& { return c[gi<D>(ngc, a, b, e)]; };
    if (order == 0) {  // src/m_aX_prolong.f90:39-108 (injection)
      const double v = P_(ic, jc, kc);
      for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
        for (int jj = 0; jj < 2; ++jj)
          for (int ii = 0; ii < 2; ++ii) {
            double& o = C_(i_f + ii, j_f + jj, k_f + kk);
            o = add ? o + v : v;
          }
    } else if (order == 1) {  // src/m_aX_prolong.f90:129-222 (2-1-1 / 1-1-1-1)
      if constexpr (D == 2) {
        const double f0 = 0.5 * P_(ic, jc, 0);
        const double flx = 0.25 * P_(ic - 1, jc, 0), fhx = 0.25 * P_(ic + 1, jc, 0);
        const double fly = 0.25 * P_(ic, jc - 1, 0), fhy = 0.25 * P_(ic, jc + 1, 0);
        double* o;
        o = &C_(i_f, j_f, 0);         *o = f0 + flx + fly + (add ? *o : 0.0);
        o = &C_(i_f + 1, j_f, 0);     *o = f0 + fhx + fly + (add ? *o : 0.0);
        o = &C_(i_f, j_f + 1, 0);     *o = f0 + flx + fhy + (add ? *o : 0.0);
        o = &C_(i_f + 1, j_f + 1, 0); *o = f0 + fhx + fhy + (add ? *o : 0.0);
      } else {
        const double f0 = 0.25 * P_(ic, jc, kc);
        const double flx = 0.25 * P_(ic - 1, jc, kc), fhx = 0.25 * P_(ic + 1, jc, kc);
        const double fly = 0.25 * P_(ic, jc - 1, kc), fhy = 0.25 * P_(ic, jc + 1, kc);
        const double flz = 0.25 * P_(ic, jc, kc - 1), fhz = 0.25 * P_(ic, jc, kc + 1);
        for (int kk = 0; kk < 2; ++kk)
          for (int jj = 0; jj < 2; ++jj)
            for (int ii = 0; ii < 2; ++ii) {
              double& o = C_(i_f + ii, j_f + jj, k_f + kk);
              o = f0 + (ii ? fhx : flx) + (jj ? fhy : fly) + (kk ? fhz : flz) + (add ? o : 0.0);
            }
      }
    } else {  // src/m_aX_prolong.f90:243-348 (quadratic)
      const double f0 = P_(ic, jc, kc);
      const double fx = 0.125 * (P_(ic + 1, jc, kc) - P_(ic - 1, jc, kc));
      const double fy = 0.125 * (P_(ic, jc + 1, kc) - P_(ic, jc - 1, kc));
      const double fxx = 0.03125 * (P_(ic - 1, jc, kc) - 2 * f0 + P_(ic + 1, jc, kc));
      const double fyy = 0.03125 * (P_(ic, jc - 1, kc) - 2 * f0 + P_(ic, jc + 1, kc));
      if constexpr (D == 2) {
        const double f2 = fxx + fyy;
        for (int jj = 0; jj < 2; ++jj)
          for (int ii = 0; ii < 2; ++ii) {
            double& o = C_(i_f + ii, j_f + jj, 0);
            const double a = ii ? f0 + fx : f0 - fx;
            o = (jj ? a + fy : a - fy) + f2 + (add ? o : 0.0);
          }
      } else {
        const double fz = 0.125 * (P_(ic, jc, kc + 1) - P_(ic, jc, kc - 1));
        const double fzz = 0.03125 * (P_(ic, jc, kc - 1) - 2 * f0 + P_(ic, jc, kc + 1));
        const double f2 = fxx + fyy + fzz;
        for (int kk = 0; kk < 2; ++kk)
          for (int jj = 0; jj < 2; ++jj)
            for (int ii = 0; ii < 2; ++ii) {
              double& o = C_(i_f + ii, j_f + jj, k_f + kk);
              const double a = ii ? f0 + fx : f0 - fx;
              const double b = jj ? a + fy : a - fy;
              o = (kk ? b + fz : b - fz) + f2 + (add ? o : 0.0);
            }
      }
    }
  }
}

// a$D_restrict_box for every child of the parents of a level,
// src/m_aX_restrict.f90:67-132: the average of the 2^D fine cells, summed in
// Fortran's column-major order starting from zero; in cylindrical trees the
// inner and outer pairs weighted at the parent's radius of index i (the
// reference's index within the child's quadrant, :90-103).
template <int D>
__global__ void k_restrict(XT t, const int* __restrict__ parents, int np, int nch, int ncp, int ncc,
                           const double* __restrict__ src, double* __restrict__ dst) {
  const int hnc = ncc / 2;
  const long long per_child = D == 2 ? (long long)hnc * hnc : (long long)hnc * hnc * hnc;
  const long long n = (long long)np * nch * per_child;
  const int ngp = ncp + 2, ngc = ncc + 2;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < n;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % per_child);
    const int ch = (int)((it / per_child) % nch);
    const int P = parents[it / per_child / nch];
    const int C = t.first_child[P] + ch;
    const int i = q % hnc + 1, j = (q / hnc) % hnc + 1, k = D == 3 ? q / (hnc * hnc) + 1 : 0;
    const int ic = i + child_off(t, C, 0, hnc), jc = j + child_off(t, C, 1, hnc);
    const int kc = D == 3 ? k + child_off(t, C, 2, hnc) : 0;
    const double* c = src + t.offg[C];
    const int i_f = 2 * i - 1, j_f = 2 * j - 1, k_f = D == 3 ? 2 * k - 1 : 0;
    if (D == 2 && t.cyl) {
      double w1, w2;
      cyl_weights(t.rmin[(size_t)P * D], t.desc[P].dr, i, w1, w2);
      double s1 = 0.0, s2 = 0.0;
      s1 = s1 + c[gi<D>(ngc, i_f, j_f, 0)];
      s1 = s1 + c[gi<D>(ngc, i_f, j_f + 1, 0)];
      s2 = s2 + c[gi<D>(ngc, i_f + 1, j_f, 0)];
      s2 = s2 + c[gi<D>(ngc, i_f + 1, j_f + 1, 0)];
      dst[t.offg[P] + gi<D>(ngp, ic, jc, kc)] = 0.25 * (w1 * s1 + w2 * s2);
      continue;
    }
    double s = 0.0;
    for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
      for (int jj = 0; jj < 2; ++jj)
        for (int ii = 0; ii < 2; ++ii) s = s + c[gi<D>(ngc, i_f + ii, j_f + jj, k_f + kk)];
    dst[t.offg[P] + gi<D>(ngp, ic, jc, kc)] = (D == 2 ? 0.25 : 0.125) * s;
  }
}

// Ghost cell (a, b) of face f (0-based) of an nc box, the adjacent interior
// cell, and the index of the neighbour's boundary cell across the face.
template <int D>
struct FaceIx {
  int g[3], a[3], n[3];
  __device__ FaceIx(int f, int nc, int u, int w) {
    const int dim = f >> 1, hi = f & 1;
    int tang[2] = {u, w};
    int e = 0;
    for (int d = 0; d < 3; ++d) {
      if (d >= D) {
        g[d] = a[d] = n[d] = 0;
      } else if (d == dim) {
        g[d] = hi ? nc + 1 : 0;
        a[d] = hi ? nc : 1;
        n[d] = hi ? 1 : nc;
      } else {
        g[d] = a[d] = n[d] = tang[e++];
      }
    }
  }
};

enum { kRbMg = 0, kRbProlong0 = 1, kRbInterp = 2, kRbInterpLim = 3 };
enum { kBcTable = 0, kBcDirichletZero = -1, kBcNeumannZero = -2 };

// a$D_gc_box on every box of one level for cell variable v: neighbours copy
// (sides_from_nb), refinement boundaries by the chosen sides_rb, physical
// boundaries by bc_to_gc with zero values or the forest's sampled sides_bc
// records. One thread per face ghost cell; the level's ghost cells are all
// independent (the sources are interior cells of the level and cells of the
// parents, which are filled first).
template <int D>
__global__ void k_gc_level(XT t, int lo, int nbx, int nc, double* __restrict__ v, int rb, int bc) {
  const int nf = D == 2 ? nc : nc * nc;
  const long long n = (long long)nbx * 2 * D * nf;
  const int ng = nc + 2, hnc = nc / 2;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < n;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % nf);
    const int f = (int)((it / nf) % (2 * D));
    const int s = lo + (int)(it / nf / (2 * D));
    const int u = q % nc + 1, w = D == 3 ? q / nc + 1 : 0;
    const FaceIx<D> F(f, nc, u, w);
    double* b = v + t.offg[s];
    const long long gpos = gi<D>(ng, F.g[0], F.g[1], F.g[2]);
    const int nbs = t.nb[s * 2 * D + f];
    const int dim = f >> 1;
    if (nbs >= 0) {  // sides_from_nb, src/m_aX_gc.f90:381-415
      b[gpos] = v[t.offg[nbs] + gi<D>(ng, F.n[0], F.n[1], F.n[2])];
    } else if (nbs == -1) {
      const int P = t.parent[s];
      int off[3] = {0, 0, 0};
      for (int d = 0; d < D; ++d) off[d] = child_off(t, s, d, hnc);
      if (rb == kRbMg || rb == kRbProlong0) {
        // a$D_gc_prolong0 (src/m_aX_gc.f90:135-151): inject the parent's cell
        // (a ghost cell of the parent in the normal direction at low faces)
        int pc[3] = {0, 0, 0};
        for (int d = 0; d < D; ++d) pc[d] = off[d] + ((F.g[d] + 1) >> 1);
        const double g0 = v[t.offg[P] + gi<D>(ng, pc[0], pc[1], pc[2])];
        if (rb == kRbProlong0) {
          b[gpos] = g0;
        } else {  // mg$D_sides_rb, src/m_aX_mg.f90:286-347
          const int dix = (f & 1) ? -1 : 1;
          const int i = F.a[0], j = F.a[1], k = F.a[2];
          auto O = [&](int a_, int b_, int c_) { return b[gi<D>(ng, a_, b_, c_)]; };
          if constexpr (D == 2) {
            if (dim == 0) {
              const int dj = -1 + 2 * (j & 1);
              b[gpos] = 0.5 * g0 + O(i, j, 0) - 0.25 * (O(i + dix, j, 0) + O(i, j + dj, 0));
            } else {
              const int di = -1 + 2 * (i & 1);
              b[gpos] = 0.5 * g0 + O(i, j, 0) - 0.25 * (O(i + di, j, 0) + O(i, j + dix, 0));
            }
          } else {
            const int di = dim == 0 ? dix : -1 + 2 * (i & 1);
            const int dj = dim == 1 ? dix : -1 + 2 * (j & 1);
            const int dk = dim == 2 ? dix : -1 + 2 * (k & 1);
            b[gpos] = 0.5 * g0 + 0.75 * O(i, j, k) - 0.25 * O(i + di, j + dj, k + dk);
          }
        }
      } else {
        // a$D_gc_interp / a$D_gc_interp_lim, src/m_aX_gc.f90:155-358: the
        // parent's neighbour across the face and the box's own first cell
        const int pn = t.nb[P * 2 * D + f];
        const double* pb = v + t.offg[pn];
        const int ix_c = (f & 1) ? 1 : nc;
        const double sixth = 1 / 6.0, third = 1 / 3.0;
        int c1[3], c2[3], c3[3];
        // tangential coarse indices: t1 = off + (x+1)/2, t2 = t1 + 1 - 2*(x&1)
        int tc1[3] = {0, 0, 0}, tc2[3] = {0, 0, 0};
        for (int d = 0; d < D; ++d)
          if (d != dim) {
            tc1[d] = off[d] + ((F.g[d] + 1) >> 1);
            tc2[d] = tc1[d] + 1 - 2 * (F.g[d] & 1);
          }
        for (int d = 0; d < 3; ++d) c1[d] = c2[d] = c3[d] = d == dim ? ix_c : tc1[d];
        const double own = b[gi<D>(ng, F.a[0], F.a[1], F.a[2])];
        double val, cv1;
        if constexpr (D == 2) {
          const int e = 1 - dim;  // the tangential direction
          c2[e] = tc2[e];
          cv1 = pb[gi<D>(ng, c1[0], c1[1], 0)];
          const double cv2 = pb[gi<D>(ng, c2[0], c2[1], 0)];
          val = 0.5 * cv1 + sixth * cv2 + third * own;
        } else {
          // first and second tangential directions (x before y before z);
          // the reference's 3-D forms vary the faster index in the second
          // term for dims 1 and 2 (j, k for x faces; i, k for y; i, j for z)
          const int e1 = dim == 0 ? 1 : 0, e2 = dim == 2 ? 1 : 2;
          if (dim == 2) {
            // z faces: c2 varies j (the slower tangential), c3 varies i
            c2[e2] = tc2[e2];
            c3[e1] = tc2[e1];
          } else {
            // x faces: c2 varies j, c3 varies k; y faces: c2 varies i, c3 varies k
            c2[e1] = tc2[e1];
            c3[e2] = tc2[e2];
          }
          cv1 = pb[gi<D>(ng, c1[0], c1[1], c1[2])];
          const double cv2 = pb[gi<D>(ng, c2[0], c2[1], c2[2])];
          const double cv3 = pb[gi<D>(ng, c3[0], c3[1], c3[2])];
          val = third * cv1 + sixth * cv2 + sixth * cv3 + third * own;
        }
        if (rb == kRbInterpLim && val > 2 * cv1) val = 2 * cv1;
        b[gpos] = val;
      }
    } else {  // physical boundary: the hook's value, then bc_to_gc (src/m_aX_gc.f90:71-132)
      const SlotDesc& d = t.desc[s];
      int code;
      double bv = 0;
      if (bc == kBcTable) {
        code = d.code[f];
        const long long o = d.nbo[f];
        if (o >= 0) bv = t.bcval[o + (D == 2 ? (u - 1) : (u - 1) + nc * (w - 1))];
      } else {
        code = bc == kBcNeumannZero ? kFaceNeumann : kFaceDirichlet;
      }
      const double x = b[gi<D>(ng, F.a[0], F.a[1], F.a[2])];
      if (code == kFaceDirichlet) {
        b[gpos] = 2.0 * bv + (-1.0) * x;
      } else {
        const double c2 = d.dr * ((f & 1) ? 1 : -1);
        b[gpos] = c2 * bv + 1.0 * x;
      }
    }
  }
}

// a$D_gc2_box on every box of a level (src/m_aX_gc.f90:420-440): the second
// layer of ghost cells per face, written to out (per box 2D faces of nf
// values, face-major, first tangential index fastest). Neighbours give their
// second cell from the face (sides2_from_nb, :443-478); refinement
// boundaries a$D_gc2_prolong1 (:481-583); physical boundaries
// a$D_bc2_neumann_zero (:586-632).
template <int D>
__global__ void k_gc2_level(XT t, const int* __restrict__ slots, int nbx, int nc, const double* __restrict__ v,
                            double* __restrict__ out) {
  const int nf = D == 2 ? nc : nc * nc;
  const long long n = (long long)nbx * 2 * D * nf;
  const int ng = nc + 2, hnc = nc / 2;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < n;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % nf);
    const int f = (int)((it / nf) % (2 * D));
    const int bi = (int)(it / nf / (2 * D));
    const int s = slots[bi];
    const int u = q % nc + 1, w = D == 3 ? q / nc + 1 : 0;
    const int dim = f >> 1, hi = f & 1;
    int tang[2] = {u, w}, c[3] = {0, 0, 0};
    {
      int e = 0;
      for (int d = 0; d < D; ++d)
        if (d != dim) c[d] = tang[e++];
    }
    const int nbs = t.nb[s * 2 * D + f];
    double val;
    if (nbs >= 0) {
      c[dim] = hi ? 2 : nc - 1;
      val = v[t.offg[nbs] + gi<D>(ng, c[0], c[1], c[2])];
    } else if (nbs == -1) {
      const int P = t.parent[s];
      const int pn = t.nb[P * 2 * D + f];
      const double* pb = v + t.offg[pn];
      const int ix = hi * (nc + 3) - 1;  // -1 or nc + 2
      int c1[3] = {0, 0, 0}, c2[3] = {0, 0, 0};
      for (int d = 0; d < D; ++d) {
        const int x = d == dim ? ix : c[d];
        // a$D_get_child_offset(box, nb): the offset on the parent's
        // neighbour, shifted by one parent width in the normal direction
        int off = child_off(t, s, d, hnc);
        if (d == dim) off -= (hi ? 1 : -1) * (t.lvl[s] > 1 ? nc : hnc);
        c1[d] = off + ((x + 1) >> 1);
        c2[d] = c1[d] + 1 - 2 * (x & 1);
      }
      auto PB = [&](int a, int b, int e) { return pb[gi<D>(ng, a, b, e)]; };
      if constexpr (D == 2) {
        val = 0.5 * PB(c1[0], c1[1], 0) + 0.25 * PB(c2[0], c1[1], 0) + 0.25 * PB(c1[0], c2[1], 0);
      } else {
        val = 0.25 * PB(c1[0], c1[1], c1[2]) + 0.25 * PB(c2[0], c1[1], c1[2]) +
              0.25 * PB(c1[0], c2[1], c1[2]) + 0.25 * PB(c1[0], c1[1], c2[2]);
      }
    } else {
      c[dim] = hi ? nc - 1 : 2;
      val = v[t.offg[s] + gi<D>(ng, c[0], c[1], c[2])];
    }
    out[it] = val;
  }
}

// a$D_consistent_fluxes for the parents of one level (src/m_aX_core.f90:
// 811-945): where a parent's neighbour across face f exists and has no
// children, the neighbour's face fluxes on that face become the average of
// the adjacent children's fine fluxes, in cylindrical trees with the radial
// weights of the neighbour's cell for the axial fluxes (:881-895). One thread
// per coarse face value.
template <int D>
__global__ void k_flux_level(XT t, const int* __restrict__ parents, int np, int nc, double* __restrict__ fc,
                             long long stride, const int* __restrict__ ifc, int nfc, long long per_var) {
  const int nch = nc / 2;
  const int nf = D == 2 ? nc : nc * nc;  // coarse face values per face
  const long long n = (long long)np * 2 * D * nf * nfc;
  const long long fb = (long long)(nc + 1) * (D == 2 ? nc : nc * nc);  // one direction's block
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < n;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % nf);
    const int f = (int)((it / nf) % (2 * D));
    const int vi = (int)((it / nf / (2 * D)) % nfc);
    const int P = parents[it / nf / (2 * D) / nfc];
    const int nbs = t.nb[P * 2 * D + f];
    if (nbs < 0 || t.first_child[nbs] >= 0) continue;
    const int dim = f >> 1, hi = f & 1;
    const int i_fine = hi ? nc + 1 : 1, i_nb = hi ? 1 : nc + 1;
    // the coarse face cell (tangential indices u, w) and the child that covers it
    const int u = q % nc + 1, w = D == 3 ? q / nc + 1 : 1;
    int tang[2] = {u, w}, cc[3] = {1, 1, 1};
    {
      int e = 0;
      for (int d = 0; d < D; ++d)
        if (d != dim) cc[d] = tang[e++];
    }
    int ch = 0;  // child-number bits: hi side in dim, the half of each tangential index
    for (int d = 0; d < D; ++d) {
      const int bit = d == dim ? hi : (cc[d] > nch ? 1 : 0);
      ch |= bit << d;
    }
    const int C = t.first_child[P] + ch;
    int fi[3] = {0, 0, 0};  // first fine index per tangential direction
    for (int d = 0; d < D; ++d)
      if (d != dim) fi[d] = 2 * (cc[d] - (cc[d] > nch ? nch : 0)) - 1;
    const double* cf = fc + (long long)ifc[vi] * per_var + (long long)C * stride + dim * fb;
    double* nf_ = fc + (long long)ifc[vi] * per_var + (long long)nbs * stride + dim * fb;
    // index of face value (x, y, z) in the dim-direction block: the normal
    // index runs 1..nc+1, the others 1..nc (x fastest)
    auto fidx = [&](int x, int y, int z) -> long long {
      const int sx = dim == 0 ? nc + 1 : nc, sy = dim == 1 ? nc + 1 : nc;
      return (long long)(x - 1) + (long long)sx * ((y - 1) + (long long)sy * (D == 3 ? z - 1 : 0));
    };
    int a[3], b[3];
    for (int d = 0; d < 3; ++d) a[d] = b[d] = (d < D) ? (d == dim ? i_fine : fi[d]) : 1;
    double val;
    if constexpr (D == 2) {
      const int e = 1 - dim;
      b[e] = a[e] + 1;
      if (dim == 1 && t.cyl) {
        double w1, w2;
        cyl_weights(t.rmin[(size_t)nbs * D], t.desc[nbs].dr, cc[0], w1, w2);
        val = 0.5 * (w1 * cf[fidx(a[0], a[1], 1)] + w2 * cf[fidx(b[0], b[1], 1)]);
      } else {
        val = 0.5 * (cf[fidx(a[0], a[1], 1)] + cf[fidx(b[0], b[1], 1)]);
      }
    } else {
      const int e1 = dim == 0 ? 1 : 0, e2 = dim == 2 ? 1 : 2;
      int a2[3] = {a[0], a[1], a[2]}, a3[3] = {a[0], a[1], a[2]}, a4[3] = {a[0], a[1], a[2]};
      a2[e1] += 1;
      a3[e2] += 1;
      a4[e1] += 1;
      a4[e2] += 1;
      val = 0.25 * (cf[fidx(a[0], a[1], a[2])] + cf[fidx(a2[0], a2[1], a2[2])] + cf[fidx(a3[0], a3[1], a3[2])] +
                    cf[fidx(a4[0], a4[1], a4[2])]);
    }
    int o[3];
    for (int d = 0; d < 3; ++d) o[d] = (d < D) ? (d == dim ? i_nb : cc[d]) : 1;
    nf_[fidx(o[0], o[1], o[2])] = val;
  }
}

// Leaf interiors of one tree gathered for output: per leaf box, cell values
// of the selected variables and the cell averages of face variables.
template <int D>
__global__ void k_gather_leaves(XT t, const int* __restrict__ slots, int nbx, int nc,
                                const double* const* __restrict__ vars, int nv, const double* __restrict__ fc,
                                long long stride, long long per_var, const int* __restrict__ ifc, int nfc,
                                double* __restrict__ out) {
  const int per = D == 2 ? nc * nc : nc * nc * nc;
  const long long ncells = (long long)nbx * per;
  const long long n = ncells * (nv + D * nfc);
  const int ng = nc + 2;
  const long long fb = (long long)(nc + 1) * (D == 2 ? nc : nc * nc);
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < n;
       it += (long long)gridDim.x * blockDim.x) {
    const long long cell = it % ncells;
    const int col = (int)(it / ncells);
    const int s = slots[cell / per];
    const int q = (int)(cell % per);
    const int i = q % nc + 1, j = (q / nc) % nc + 1, k = D == 3 ? q / (nc * nc) + 1 : 1;
    if (col < nv) {
      out[it] = vars[col][t.offg[s] + gi<D>(ng, i, j, D == 3 ? k : 0)];
    } else {
      const int vi = (col - nv) / D, dim = (col - nv) % D;
      const double* f = fc + (long long)ifc[vi] * per_var + (long long)s * stride + dim * fb;
      const int sx = dim == 0 ? nc + 1 : nc, sy = dim == 1 ? nc + 1 : nc;
      auto fidx = [&](int x, int y, int z) -> long long {
        return (long long)(x - 1) + (long long)sx * ((y - 1) + (long long)sy * (D == 3 ? z - 1 : 0));
      };
      const int i2 = i + (dim == 0), j2 = j + (dim == 1), k2 = k + (dim == 2);
      // 0.5_dp * sum(fx(i:i+1, j, k)): the Fortran sum from zero
      double sum = 0.0;
      sum = sum + f[fidx(i, j, k)];
      sum = sum + f[fidx(i2, j2, k2)];
      out[it] = 0.5 * sum;
    }
  }
}

}  // namespace xdev

namespace {

int grid_of(long long items, int n_sm) {
  return (int)std::max(1LL, std::min((items + 255) / 256, (long long)n_sm * 8));
}

// Slot tables of the utilities on the device (first use).
int ensure_tables(Forest& F, std::string& err) {
  if (F.d_nb) return AFV_OK;
  const Plan& p = F.plan;
  std::vector<int> qd(p.qd);
  auto up = [&](int** d, const std::vector<int>& h) -> bool {
    if (cudaMallocAsync((void**)d, sizeof(int) * std::max<size_t>(1, h.size()), F.stream) != cudaSuccess) return false;
    return cudaMemcpyAsync(*d, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, F.stream) == cudaSuccess;
  };
  if (!up(&F.d_nb, p.nb) || !up(&F.d_lvl, p.lvl) || !up(&F.d_qd, qd))
    return err = "device allocation of the slot tables failed", AFV_ERR_NOMEM;
  if (cudaStreamSynchronize(F.stream) != cudaSuccess) return err = "slot table upload failed", AFV_ERR_CUDA;
  return AFV_OK;
}

xdev::XT tables(const Forest& F) {
  xdev::XT t;
  t.nb = F.d_nb;
  t.parent = F.meta.parent;
  t.first_child = F.meta.first_child;
  t.lvl = F.d_lvl;
  t.qd = F.d_qd;
  t.offg = F.meta.offg;
  t.desc = F.meta.desc;
  t.bcval = F.meta.bcval;
  t.rmin = F.meta.rmin;
  t.cyl = F.plan.cyl;
  return t;
}

int finish(Forest& F, std::string& err, const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return err = std::string(where) + ": " + cudaGetErrorString(e), AFV_ERR_CUDA;
  return AFV_OK;
}

// Ghosted cell variable iv (the rhs has no ghost cells in this layout).
int ghosted_var(Forest& F, int iv, double** out, std::string& err) {
  if (iv == AFV_RHS) return err = "rhs has no ghost cells on the device", AFV_ERR_UNSUPPORTED;
  double* v = F.var_ptr(iv);
  if (!v) return err = "unknown variable", AFV_ERR_INVALID;
  *out = v;
  return AFV_OK;
}

}  // namespace

int forest_add_vars(Forest& F, int n_cc, int n_fc, std::string& err) {
  if (n_cc < 0 || n_fc < 0 || n_cc > 64 || n_fc > 64) return err = "bad variable counts", AFV_ERR_INVALID;
  if (n_fc && F.n_fc) return err = "face variables were added already", AFV_ERR_STATE;
  const Plan& p = F.plan;
  for (int k = 0; k < n_cc; ++k) {
    double* v = nullptr;
    if (cudaMallocAsync((void**)&v, sizeof(double) * std::max(1LL, p.n_elem_g), F.stream) != cudaSuccess)
      return err = "device allocation of a cell variable failed", AFV_ERR_NOMEM;
    cudaMemsetAsync(v, 0, sizeof(double) * p.n_elem_g, F.stream);
    F.xcc.push_back(v);
    F.bytes += sizeof(double) * p.n_elem_g;
  }
  if (n_fc) {
    long long fb = (long long)(p.nc + 1) * (p.dim == 2 ? p.nc : p.nc * p.nc);
    F.fc_stride = p.dim * fb;
    const long long n = (long long)n_fc * p.n_slots * F.fc_stride;
    if (cudaMallocAsync((void**)&F.fc, sizeof(double) * std::max(1LL, n), F.stream) != cudaSuccess)
      return err = "device allocation of the face variables failed", AFV_ERR_NOMEM;
    cudaMemsetAsync(F.fc, 0, sizeof(double) * n, F.stream);
    F.n_fc = n_fc;
    F.bytes += sizeof(double) * n;
  }
  if (cudaStreamSynchronize(F.stream) != cudaSuccess) return finish(F, err, "add_vars");
  return AFV_OK;
}

// Face variable ifc of one tree to or from the host: per box in the host
// exchange order, D blocks (fx(1:nc+1,1:nc[,1:nc]), fy(...), fz(...)), each
// with x fastest, of the box's own n_cell.
int forest_fc_exchange(Forest& F, int t, int ifc, double* host, bool to_dev, std::string& err) {
  const Plan& p = F.plan;
  if (t < 0 || t >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  if (ifc < 0 || ifc >= F.n_fc) return err = "unknown face variable", AFV_ERR_INVALID;
  const int D = p.dim;
  const long long per_var = (long long)p.n_slots * F.fc_stride;
  long long off = 0;
  for (int s : p.host_order[t]) {
    const int nc = p.nc_at(p.lvl[s]);
    const long long fb = (long long)(nc + 1) * (D == 2 ? nc : nc * nc);
    const long long full_fb = F.fc_stride / D;
    for (int d = 0; d < D; ++d) {
      double* dev = F.fc + ifc * per_var + (long long)s * F.fc_stride + d * full_fb;
      cudaMemcpyAsync(to_dev ? (void*)dev : (void*)(host + off), to_dev ? (const void*)(host + off) : (const void*)dev,
                      sizeof(double) * fb, to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, F.stream);
      off += fb;
    }
  }
  if (cudaStreamSynchronize(F.stream) != cudaSuccess) return finish(F, err, "face exchange");
  return finish(F, err, "face exchange");
}

long long forest_fc_count(const Forest& F, int t) {
  const Plan& p = F.plan;
  long long n = 0;
  for (int s : p.host_order[t]) {
    const int nc = p.nc_at(p.lvl[s]);
    n += (long long)p.dim * (nc + 1) * (p.dim == 2 ? nc : nc * nc);
  }
  return n;
}

// a$D_prolong{order}_from on every parent of level lp (all trees).
int forest_prolong(Forest& F, int lp, int iv, int iv_to, int order, int add, std::string& err) {
  const Plan& p = F.plan;
  if (order < 0 || order > 2) return err = "prolongation order must be 0, 1 or 2", AFV_ERR_INVALID;
  if (lp < p.min_lvl || lp >= p.max_lvl) return err = "level out of range", AFV_ERR_INVALID;
  double *src, *dst;
  if (int rc = ghosted_var(F, iv, &src, err)) return rc;
  if (int rc = ghosted_var(F, iv_to, &dst, err)) return rc;
  if (int rc = ensure_tables(F, err)) return rc;
  const int np = F.n_parents(lp);
  if (!np) return AFV_OK;
  const int nch = lp >= 1 ? (1 << p.dim) : 1;
  const int ncp = p.nc_at(lp), ncc = p.nc_at(lp + 1);
  const long long items = (long long)np * nch * (p.dim == 2 ? (ncc / 2) * (ncc / 2) : (ncc / 2) * (ncc / 2) * (ncc / 2));
  const xdev::XT t = tables(F);
  if (p.dim == 2)
    xdev::k_prolong<2><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, F.parents_list(lp), np, nch, ncp, ncc, src, dst,
                                                                     order, add);
  else
    xdev::k_prolong<3><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, F.parents_list(lp), np, nch, ncp, ncc, src, dst,
                                                                     order, add);
  ++F.n_launches;
  return finish(F, err, "prolong");
}

// a$D_restrict_tree(tree, iv, iv_to): every level's parents from the finest
// down.
int forest_restrict_tree(Forest& F, int iv, int iv_to, std::string& err) {
  const Plan& p = F.plan;
  double *src, *dst;
  if (int rc = ghosted_var(F, iv, &src, err)) return rc;
  if (int rc = ghosted_var(F, iv_to, &dst, err)) return rc;
  if (int rc = ensure_tables(F, err)) return rc;
  const xdev::XT t = tables(F);
  for (int lp = p.max_lvl - 1; lp >= p.min_lvl; --lp) {
    const int np = F.n_parents(lp);
    if (!np) continue;
    const int nch = lp >= 1 ? (1 << p.dim) : 1;
    const int ncp = p.nc_at(lp), ncc = p.nc_at(lp + 1);
    const long long h = ncc / 2;
    const long long items = (long long)np * nch * (p.dim == 2 ? h * h : h * h * h);
    if (p.dim == 2)
      xdev::k_restrict<2><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, F.parents_list(lp), np, nch, ncp, ncc, src, dst);
    else
      xdev::k_restrict<3><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, F.parents_list(lp), np, nch, ncp, ncc, src, dst);
    ++F.n_launches;
  }
  return finish(F, err, "restrict_tree");
}

// a$D_gc_tree(tree, iv, subr_rb, subr_bc): levels coarse to fine.
int forest_gc_tree_var(Forest& F, int iv, int rb, int bc, std::string& err) {
  const Plan& p = F.plan;
  if (rb < xdev::kRbMg || rb > xdev::kRbInterpLim) return err = "unknown refinement-boundary method", AFV_ERR_INVALID;
  if (bc != xdev::kBcTable && bc != xdev::kBcDirichletZero && bc != xdev::kBcNeumannZero)
    return err = "unknown boundary method", AFV_ERR_INVALID;
  double* v;
  if (int rc = ghosted_var(F, iv, &v, err)) return rc;
  if (int rc = ensure_tables(F, err)) return rc;
  const xdev::XT t = tables(F);
  for (int l = p.min_lvl; l <= p.max_lvl; ++l) {
    const int nbx = F.lvl_n(l);
    if (!nbx) continue;
    const int nc = p.nc_at(l);
    const long long items = (long long)nbx * 2 * p.dim * (p.dim == 2 ? nc : nc * nc);
    const int lo = p.lvl_lo[p.L(l)];
    if (p.dim == 2)
      xdev::k_gc_level<2><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, lo, nbx, nc, v, rb, bc);
    else
      xdev::k_gc_level<3><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, lo, nbx, nc, v, rb, bc);
    ++F.n_launches;
  }
  return finish(F, err, "gc_tree");
}

// a$D_gc2_box on the boxes of one tree on one level, in the tree's level-list
// order; out receives per box 2D faces of nc^(D-1) values.
int forest_gc2_level(Forest& F, int tree, int lvl, int iv, double* host_out, long long n_out, std::string& err) {
  const Plan& p = F.plan;
  if (tree < 0 || tree >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  if (lvl < 1 || lvl > p.max_lvl) return err = "level out of range (levels >= 1)", AFV_ERR_INVALID;
  double* v;
  if (int rc = ghosted_var(F, iv, &v, err)) return rc;
  if (int rc = ensure_tables(F, err)) return rc;
  std::vector<int> slots;
  for (int s : p.host_order[tree])
    if (p.lvl[s] == lvl) slots.push_back(s);
  const int nc = p.nc_at(lvl);
  const long long per = 2LL * p.dim * (p.dim == 2 ? nc : nc * nc);
  if (n_out != (long long)slots.size() * per) return err = "output size does not match the level", AFV_ERR_INVALID;
  if (slots.empty()) return AFV_OK;
  int* d_slots = nullptr;
  double* d_out = nullptr;
  if (cudaMallocAsync((void**)&d_slots, sizeof(int) * slots.size(), F.stream) != cudaSuccess ||
      cudaMallocAsync((void**)&d_out, sizeof(double) * n_out, F.stream) != cudaSuccess) {
    if (d_slots) cudaFreeAsync(d_slots, F.stream);
    return err = "device allocation failed", AFV_ERR_NOMEM;
  }
  cudaMemcpyAsync(d_slots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice, F.stream);
  const xdev::XT t = tables(F);
  if (p.dim == 2)
    xdev::k_gc2_level<2><<<grid_of(n_out, F.n_sm), 256, 0, F.stream>>>(t, d_slots, (int)slots.size(), nc, v, d_out);
  else
    xdev::k_gc2_level<3><<<grid_of(n_out, F.n_sm), 256, 0, F.stream>>>(t, d_slots, (int)slots.size(), nc, v, d_out);
  ++F.n_launches;
  cudaMemcpyAsync(host_out, d_out, sizeof(double) * n_out, cudaMemcpyDeviceToHost, F.stream);
  cudaFreeAsync(d_slots, F.stream);
  cudaFreeAsync(d_out, F.stream);
  if (cudaStreamSynchronize(F.stream) != cudaSuccess) return finish(F, err, "gc2");
  return finish(F, err, "gc2");
}

// a$D_consistent_fluxes(tree, f_ixs): the parents of every level, coarse to fine.
int forest_consistent_fluxes(Forest& F, int n, const int* f_ixs, std::string& err) {
  const Plan& p = F.plan;
  if (!F.n_fc) return err = "the forest has no face variables", AFV_ERR_STATE;
  if (n <= 0 || !f_ixs) return err = "no face variables given", AFV_ERR_INVALID;
  for (int k = 0; k < n; ++k)
    if (f_ixs[k] < 0 || f_ixs[k] >= F.n_fc) return err = "unknown face variable", AFV_ERR_INVALID;
  if (int rc = ensure_tables(F, err)) return rc;
  int* d_ix = nullptr;
  if (cudaMallocAsync((void**)&d_ix, sizeof(int) * n, F.stream) != cudaSuccess)
    return err = "device allocation failed", AFV_ERR_NOMEM;
  cudaMemcpyAsync(d_ix, f_ixs, sizeof(int) * n, cudaMemcpyHostToDevice, F.stream);
  const xdev::XT t = tables(F);
  const long long per_var = (long long)p.n_slots * F.fc_stride;
  for (int lp = p.min_lvl; lp <= p.max_lvl - 1; ++lp) {
    const int np = F.n_parents(lp);
    if (!np || lp < 1) continue;  // sub-level boxes have one child: no refinement faces
    const int nc = p.nc_at(lp);
    const long long items = (long long)np * 2 * p.dim * (p.dim == 2 ? nc : nc * nc) * n;
    if (p.dim == 2)
      xdev::k_flux_level<2><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, F.parents_list(lp), np, nc, F.fc,
                                                                          F.fc_stride, d_ix, n, per_var);
    else
      xdev::k_flux_level<3><<<grid_of(items, F.n_sm), 256, 0, F.stream>>>(t, F.parents_list(lp), np, nc, F.fc,
                                                                          F.fc_stride, d_ix, n, per_var);
    ++F.n_launches;
  }
  cudaFreeAsync(d_ix, F.stream);
  if (cudaStreamSynchronize(F.stream) != cudaSuccess) return finish(F, err, "consistent_fluxes");
  return finish(F, err, "consistent_fluxes");
}

namespace {

// The m_vtk.f90 writer's pieces: XML lines into the file, raw arrays (each
// preceded by its byte count as a 4-byte integer) into the appended block.
struct VtuWriter {
  std::string head;
  std::vector<char> raw;
  int indent = 0;
  long long offset = 0;
  void line(const std::string& s) { head += std::string(indent, ' ') + s + "\n"; }
  void open(const std::string& n) {
    line("<" + n + ">");
    indent += 2;
  }
  void close(const std::string& n) {
    indent -= 2;
    line("</" + n + ">");
  }
  void append(const void* p, long long bytes) {
    const int nb = (int)bytes;
    const char* c = reinterpret_cast<const char*>(&nb);
    raw.insert(raw.end(), c, c + 4);
    const char* d = reinterpret_cast<const char*>(p);
    raw.insert(raw.end(), d, d + bytes);
    offset += 4 + bytes;
  }
};

// Text of a real or integer field value (the reference writes these with
// Fortran list-directed output, whose exact spacing is compiler-specific).
std::string num_text(double x) {
  char b[64];
  std::snprintf(b, sizeof b, "%.17E", x);
  return b;
}

}  // namespace

// a$D_write_vtk: leaves of levels 1..highest of one tree, cell variables and
// cell averages of face variables, as a VTK unstructured grid (.vtu) with
// appended raw data in the m_vtk.f90 layout.
int forest_write_vtk(Forest& F, int tree, const char* filename, int n_cycle, double time, int n_cc, const int* ixs_cc,
                     const char* const* cc_names, int n_fcv, const int* ixs_fc, const char* const* fc_names,
                     const char* dir, std::string& err) {
  const Plan& p = F.plan;
  const int D = p.dim;
  if (tree < 0 || tree >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  if (!filename || n_cc < 0 || n_fcv < 0 || (n_cc && (!ixs_cc || !cc_names)) || (n_fcv && (!ixs_fc || !fc_names)))
    return err = "bad arguments", AFV_ERR_INVALID;
  std::vector<const double*> vars;
  for (int k = 0; k < n_cc; ++k) {
    double* v = F.var_ptr(ixs_cc[k]);
    if (!v || ixs_cc[k] == AFV_RHS) return err = "cell variable not writable (unknown, or rhs)", AFV_ERR_INVALID;
    vars.push_back(v);
  }
  for (int k = 0; k < n_fcv; ++k)
    if (ixs_fc[k] < 0 || ixs_fc[k] >= F.n_fc) return err = "unknown face variable", AFV_ERR_INVALID;
  if (int rc = ensure_tables(F, err)) return rc;
  // leaves of levels 1 .. highest in lvls(lvl)%leaves order (ids order)
  std::vector<int> leaves;
  std::vector<int> order = p.host_order[tree];
  for (int l = 1; l <= p.tree_highest[tree]; ++l)
    for (int s : order)
      if (p.lvl[s] == l && p.first_child[s] < 0) leaves.push_back(s);
  const int nc = p.nc;
  const int bn = nc + 1;
  const long long per = D == 2 ? (long long)nc * nc : (long long)nc * nc * nc;
  const long long nodes_per_box = D == 2 ? (long long)bn * bn : (long long)bn * bn * bn;
  const long long n_grids = (long long)leaves.size();
  const long long n_cells = per * n_grids, n_nodes = nodes_per_box * n_grids;
  const int ncol = n_cc + D * n_fcv;
  std::vector<double> cols((size_t)(n_cells * ncol));
  if (n_cells && ncol) {
    int* d_slots = nullptr;
    const double** d_vars = nullptr;
    int* d_ifc = nullptr;
    double* d_out = nullptr;
    bool ok = cudaMallocAsync((void**)&d_slots, sizeof(int) * leaves.size(), F.stream) == cudaSuccess &&
              cudaMallocAsync((void**)&d_vars, sizeof(double*) * std::max(1, n_cc), F.stream) == cudaSuccess &&
              cudaMallocAsync((void**)&d_ifc, sizeof(int) * std::max(1, n_fcv), F.stream) == cudaSuccess &&
              cudaMallocAsync((void**)&d_out, sizeof(double) * cols.size(), F.stream) == cudaSuccess;
    if (ok) {
      cudaMemcpyAsync(d_slots, leaves.data(), sizeof(int) * leaves.size(), cudaMemcpyHostToDevice, F.stream);
      if (n_cc) cudaMemcpyAsync(d_vars, vars.data(), sizeof(double*) * n_cc, cudaMemcpyHostToDevice, F.stream);
      if (n_fcv) cudaMemcpyAsync(d_ifc, ixs_fc, sizeof(int) * n_fcv, cudaMemcpyHostToDevice, F.stream);
      const xdev::XT t = tables(F);
      const long long per_var = (long long)p.n_slots * F.fc_stride;
      if (D == 2)
        xdev::k_gather_leaves<2><<<grid_of((long long)cols.size(), F.n_sm), 256, 0, F.stream>>>(
            t, d_slots, (int)n_grids, nc, d_vars, n_cc, F.fc, F.fc_stride, per_var, d_ifc, n_fcv, d_out);
      else
        xdev::k_gather_leaves<3><<<grid_of((long long)cols.size(), F.n_sm), 256, 0, F.stream>>>(
            t, d_slots, (int)n_grids, nc, d_vars, n_cc, F.fc, F.fc_stride, per_var, d_ifc, n_fcv, d_out);
      ++F.n_launches;
      cudaMemcpyAsync(cols.data(), d_out, sizeof(double) * cols.size(), cudaMemcpyDeviceToHost, F.stream);
    }
    for (void* q : {(void*)d_slots, (void*)d_vars, (void*)d_ifc, (void*)d_out})
      if (q) cudaFreeAsync(q, F.stream);
    if (cudaStreamSynchronize(F.stream) != cudaSuccess || !ok) return finish(F, err, "write_vtk");
  }
  // geometry: node coordinates of every leaf (r_min + (i-1) dr), as 4-byte
  // floats with three components
  std::vector<float> coords((size_t)(3 * n_nodes), 0.0f);
  std::vector<int> connects((size_t)((1 << D) * n_cells)), offsets((size_t)n_cells), types((size_t)n_cells, D == 2 ? 8 : 11);
  for (long long g = 0; g < n_grids; ++g) {
    const int s = leaves[(size_t)g];
    const double dr = p.dr[s];
    const double* rmin = &p.r_min[(size_t)s * D];
    const long long node0 = g * nodes_per_box, cell0 = g * per;
    for (int k = 0; k < (D == 3 ? bn : 1); ++k)
      for (int j = 0; j < bn; ++j)
        for (int i = 0; i < bn; ++i) {
          const long long nix = node0 + i + (long long)bn * (j + (long long)bn * k);
          const int ijk[3] = {i, j, k};
          for (int d = 0; d < D; ++d) coords[(size_t)(3 * nix + d)] = (float)(rmin[d] + ijk[d] * dr);
        }
    const long long bn2 = (long long)bn * bn;
    for (int k = 0; k < (D == 3 ? nc : 1); ++k)
      for (int j = 0; j < nc; ++j)
        for (int i = 0; i < nc; ++i) {
          const long long cix = cell0 + i + (long long)nc * (j + (long long)nc * k);  // 0-based
          const long long nix = node0 + (long long)k * bn2 + (long long)j * bn + i;
          offsets[(size_t)cix] = (int)((1 << D) * (cix + 1));
          int* cn = &connects[(size_t)((1 << D) * cix)];
          cn[0] = (int)nix;
          cn[1] = (int)(nix + 1);
          cn[2] = (int)(nix + bn);
          cn[3] = (int)(nix + bn + 1);
          if (D == 3) {
            cn[4] = (int)(nix + bn2);
            cn[5] = (int)(nix + bn2 + 1);
            cn[6] = (int)(nix + bn2 + bn);
            cn[7] = (int)(nix + bn2 + bn + 1);
          }
        }
  }
  std::vector<std::string> names;
  for (int k = 0; k < n_cc; ++k) names.push_back(cc_names[k]);
  const bool cyl = D == 2 && F.plan.cyl;  // a$D_write_vtk names r, z in cylindrical trees
  const char* sfx[3] = {cyl ? "_r" : "_x", cyl ? "_z" : "_y", "_z"};
  for (int k = 0; k < n_fcv; ++k)
    for (int d = 0; d < D; ++d) names.push_back(std::string(fc_names[k]) + sfx[d]);
  // the file, in the order of vtk_ini_xml .. vtk_end_xml
  VtuWriter w;
  w.head = "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  w.indent = 2;
  w.open("UnstructuredGrid");
  w.open("FieldData");
  w.line("<DataArray type=\"Float64\" Name=\"TIME\" NumberOfTuples=\"1\" format=\"ascii\">");
  w.indent += 2;
  w.line(num_text(time));
  w.close("DataArray");
  w.line("<DataArray type=\"Int32\" Name=\"CYCLE\" NumberOfTuples=\"1\" format=\"ascii\">");
  w.indent += 2;
  w.line(std::to_string(n_cycle));
  w.close("DataArray");
  w.close("FieldData");
  w.line("<Piece NumberOfPoints=\"" + std::to_string(n_nodes) + "\" NumberOfCells=\"" + std::to_string(n_cells) + "\">");
  w.indent += 2;
  w.open("Points");
  w.line("<DataArray type=\"Float32\" NumberOfComponents=\"3\" Name=\"Points\" format=\"appended\" offset=\"" +
         std::to_string(w.offset) + "\"/>");
  w.append(coords.data(), (long long)coords.size() * 4);
  w.close("Points");
  w.open("Cells");
  w.line("<DataArray type=\"Int32\" Name=\"connectivity\" format=\"appended\" offset=\"" + std::to_string(w.offset) +
         "\"/>");
  w.append(connects.data(), (long long)connects.size() * 4);
  w.line("<DataArray type=\"Int32\" Name=\"offsets\" format=\"appended\" offset=\"" + std::to_string(w.offset) + "\"/>");
  w.append(offsets.data(), (long long)offsets.size() * 4);
  w.line("<DataArray type=\"Int32\" Name=\"types\" format=\"appended\" offset=\"" + std::to_string(w.offset) + "\"/>");
  w.append(types.data(), (long long)types.size() * 4);
  w.close("Cells");
  w.open("CellData");
  for (int c = 0; c < ncol; ++c) {
    w.line("<DataArray type=\"Float64\" Name=\"" + names[(size_t)c] +
           "\" NumberOfComponents=\"1\" format=\"appended\" offset=\"" + std::to_string(w.offset) + "\"/>");
    w.append(cols.data() + (size_t)c * n_cells, n_cells * 8);
  }
  w.close("CellData");
  w.close("Piece");
  w.close("UnstructuredGrid");
  std::string path = std::string(filename) + ".vtu";
  if (dir && dir[0]) {
    std::string d(dir);
    path = (d.back() == '/' ? d : d + "/") + path;
  }
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return err = "cannot open " + path, AFV_ERR_INVALID;
  bool ok = std::fwrite(w.head.data(), 1, w.head.size(), fp) == w.head.size();
  std::string ad = std::string(w.indent, ' ') + "<AppendedData encoding=\"raw\">\n_";
  ok = ok && std::fwrite(ad.data(), 1, ad.size(), fp) == ad.size();
  ok = ok && (w.raw.empty() || std::fwrite(w.raw.data(), 1, w.raw.size(), fp) == w.raw.size());
  std::string tail = "\n" + std::string(w.indent, ' ') + "</AppendedData>\n</VTKFile>\n";
  ok = ok && std::fwrite(tail.data(), 1, tail.size(), fp) == tail.size();
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return err = "writing " + path + " failed", AFV_ERR_INVALID;
  return AFV_OK;
}

}  // namespace afv
