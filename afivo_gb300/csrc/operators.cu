// Operator variants behind the same FAS V-cycle (FP64): the variable-
// coefficient Laplacian div(eps grad phi) of mg$D_box_gsrb_lpld,
// mg$D_box_lpld and mg$D_box_corr_lpld (src/m_aX_mg.f90:810-985), their
// cylindrical forms mg2_box_*_clpl / _clpld (:1323-1443), the level-set
// operators for internal boundaries mg$D_box_*_lpllsf with their masked
// restriction (:987-1321), and the per-box dispatch of mg$D_auto_gsrb / _op /
// _corr / _rstr with the tags of mg$D_set_box_tag (:562-706). In cylindrical
// trees every operator restricts with the weights of a2_restrict_box
// (src/m_aX_restrict.f90:90-103).
//
// The schedule is the reference's, operator by operator: every half-sweep is
// followed by a ghost fill of its level (gsrb_boxes, src/m_aX_mg.f90:
// 397-420), update_coarse restricts the residual and phi (:424-480), and
// correct_children forms tmp = phi - tmp on the parents before the children
// take their correction (:368-395). Each kernel takes one thread per updated
// cell and keeps the reference's expression order, so results are
// bit-identical to the reference's routines (-fmad=false). The constant-
// coefficient Cartesian solver keeps its own fused kernels (solver.cu); this
// path is taken only for the other operators and for cylindrical trees.
#include <algorithm>
#include <string>
#include <type_traits>
#include <vector>

#include "afivo_gb300.h"
#include "forest.hpp"
#include "kernels.cuh"

namespace afv {
namespace opdev {

using dev::BoxSet;
using dev::Geo;
using dev::Meta;

enum { kTagNormal = 1, kTagLsf = 2, kTagCeps = 3, kTagVeps = 4 };  // mg_*_box
enum { kLpl = 0, kLpld = 1, kClpl = 2, kClpld = 3, kLsf = 4 };     // operator of a box

// What the kernels need to know about the forest's operator.
struct Op {
  int op;                 // AFV_OP_*
  int cyl;                // cylindrical tree (2-D)
  const int* tags;        // [slot] mg_*_box (auto dispatch)
  const double* eps;      // ghosted eps (or any valid array when unused)
  const double* lsf;      // ghosted level set function
  const double* bval;     // ghosted boundary value at the interface
  const int* ix;          // [slot*D + d]
  const double* rmin;     // [slot*D + d]
  const double* coef;     // lpld face weights eps_0 eps / (eps_0 + eps), [(offi + q) * 2D + f], or null
};

// The operator a box takes (mg%box_* hooks, or the auto dispatch by tag).
__device__ __forceinline__ int kind_of(const Op& o, int s) {
  switch (o.op) {
    case AFV_OP_LPL: return kLpl;
    case AFV_OP_LPLD: return kLpld;
    case AFV_OP_CLPL: return kClpl;
    case AFV_OP_CLPLD: return kClpld;
    case AFV_OP_LPLLSF: return kLsf;
  }
  const int t = o.tags[s];
  if (t == kTagLsf) return kLsf;
  if (t == kTagNormal) return o.cyl ? kClpl : kLpl;
  return o.cyl ? kClpld : kLpld;
}

// Offsets of the 2D face neighbours of a cell in a ghosted box, in the
// reference's order: (i-1), (i+1), (j-1), (j+1)[, (k-1), (k+1)].
template <int D, int NC>
__device__ __forceinline__ int nb_off(int k) {
  constexpr int NG = NC + 2;
  const int step = k < 2 ? 1 : (k < 4 ? NG : NG * NG);
  return (k & 1) ? step : -step;
}

// Radial factors of the cylindrical operators at interior index i of a box:
// [i+ioff-1, i+ioff] / (i+ioff-0.5), ioff = (ix(1)-1) * nc.
__device__ __forceinline__ void rfac(int i, int ioff, double& r1, double& r2) {
  r1 = (i + ioff - 1) / (i + ioff - 0.5);
  r2 = (i + ioff) / (i + ioff - 0.5);
}

// x / y. When y is a power of two whose reciprocal is a normal number, x
// times that (exact) reciprocal: the same correctly rounded quotient without
// a division. The level-set and variable-coefficient formulas divide by 2 or
// 4 away from interfaces and eps jumps (distances 1, equal eps), and GB300's
// FP64 pipe makes each division costly.
__device__ __forceinline__ double qdiv(double x, double y) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(y);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if ((b & 0xfffffffffffffull) == 0 && e >= 1 && e <= 2045)
    return x * __longlong_as_double((long long)((b & 0x8000000000000000ull) | ((unsigned long long)(2046 - e) << 52)));
  return x / y;
}

// lsf_dist_val (src/m_aX_mg.f90:993-1019): distance (0..1) to a neighbour and
// the value there, or at the interface when the level set changes sign
// between (boundary values interpolated).
__device__ __forceinline__ void lsf_dist_val(double la, double ba, double lb, double ub, double bb, double& dist,
                                             double& val) {
  if (la * lb < 0) {
    dist = la / (la - lb);
    val = ba * (1 - dist) + bb * dist;
  } else {
    dist = 1;
    val = ub;
  }
}

template <int D, int NC>
__device__ __forceinline__ void lsf_stencil(const double* u, const double* l, const double* bv, int c, double* dd,
                                            double* val) {
#pragma unroll
  for (int k = 0; k < 2 * D; ++k) {
    const int o = nb_off<D, NC>(k);
    lsf_dist_val(l[c], bv[c], l[c + o], u[c + o], bv[c + o], dd[k], val[k]);
  }
}

// L phi at ghosted index c (interior index i along x) of slot s, box offset
// g: mg$D_box_lpl, mg$D_box_lpld, mg2_box_clpl, mg2_box_clpld, mg$D_box_lpllsf.
template <int D, int NC>
__device__ __forceinline__ double op_at(const Op& o, int kind, const double* __restrict__ phi, long long g, int s,
                                        int c, int i, double inv_dr_sq, long long qi) {
  const double* u = phi + g;
  constexpr int NG = NC + 2;
  switch (kind) {
    case kLpl:
      if constexpr (D == 2)
        return inv_dr_sq * (u[c - 1] + u[c + 1] + u[c - NG] + u[c + NG] - 4 * u[c]);
      else
        return inv_dr_sq * (u[c - 1] + u[c + 1] + u[c - NG] + u[c + NG] + u[c - NG * NG] + u[c + NG * NG] - 6 * u[c]);
    case kClpl: {
      double r1, r2;
      rfac(i, (o.ix[(size_t)s * D] - 1) * NC, r1, r2);
      return (r1 * u[c - 1] + r2 * u[c + 1] + u[c - NG] + u[c + NG] - 4 * u[c]) * inv_dr_sq;
    }
    case kLsf: {
      double dd[6], val[6];
      lsf_stencil<D, NC>(u, o.lsf + g, o.bval + g, c, dd, val);
      const double f0 = u[c];
      double r = qdiv(dd[1] * val[0] + dd[0] * val[1] - (dd[0] + dd[1]) * f0, (dd[0] + dd[1]) * dd[0] * dd[1]) +
                 qdiv(dd[3] * val[2] + dd[2] * val[3] - (dd[2] + dd[3]) * f0, (dd[2] + dd[3]) * dd[2] * dd[3]);
      if constexpr (D == 3)
        r = r + qdiv(dd[5] * val[4] + dd[4] * val[5] - (dd[4] + dd[5]) * f0, (dd[4] + dd[5]) * dd[4] * dd[5]);
      return 2 * inv_dr_sq * r;
    }
    default: {  // kLpld, kClpld
      const double* e = o.eps + g;
      const double u0 = u[c], a0 = e[c];
      const bool cyl = kind == kClpld;
      if (!cyl && o.coef) {  // the face weights of k_coef: the values of the division below
        const double* w = o.coef + qi * (2 * D);
        double sum = 0.0;
#pragma unroll
        for (int k = 0; k < 2 * D; ++k) sum = sum + w[k] * (u[c + nb_off<D, NC>(k)] - u0);
        return inv_dr_sq * 2 * sum;
      }
      double r1 = 1, r2 = 1;
      if (cyl) rfac(i, (o.ix[(size_t)s * D] - 1) * NC, r1, r2);
      double sum = 0.0;
#pragma unroll
      for (int k = 0; k < 2 * D; ++k) {
        const int of = nb_off<D, NC>(k);
        const double a = e[c + of];
        if (cyl) {
          const double rf = k == 0 ? r1 : k == 1 ? r2 : 1.0;
          sum = sum + qdiv(rf * a0 * a, a0 + a) * (u[c + of] - u0);
        } else {
          sum = sum + qdiv(a0 * a, a0 + a) * (u[c + of] - u0);
        }
      }
      return inv_dr_sq * 2 * sum;
    }
  }
}

// mg$D_set_box_tag (src/m_aX_mg.f90:672-706): min and max of the level set
// and of eps over the whole box, ghost cells included, one warp per box. A box
// that would take two tags sets *conflict.
template <int D, int NC>
__global__ void k_tags(BoxSet bs, const long long* __restrict__ offg, const double* __restrict__ eps,
                       const double* __restrict__ lsf, int* __restrict__ tags, int* __restrict__ conflict) {
  using G = Geo<D, NC>;
  const int lane = threadIdx.x & 31;
  const int warps = (int)(gridDim.x * blockDim.x) >> 5;
  for (int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < bs.n; b += warps) {
    const int s = bs.lo + b;
    bool is_lsf = false, is_eps = false, is_deps = false;
    for (int which = 0; which < 2; ++which) {
      const double* base = which ? eps : lsf;
      if (!base) continue;
      const double* e = base + offg[s];
      double mn = e[0], mx = e[0];
      for (int q = lane; q < G::SG; q += 32) {
        mn = fmin(mn, e[q]);
        mx = fmax(mx, e[q]);
      }
      for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      }
      if (which) {
        is_deps = mx > mn;
        is_eps = !is_deps && (mn < 1 || mn > 1);
      } else {
        is_lsf = mn * mx < 0;
      }
    }
    if (lane == 0) {
      int t = kTagNormal;
      if (is_lsf) t = kTagLsf;
      if (is_eps) t = kTagCeps;
      if (is_deps) t = kTagVeps;
      tags[s] = t;
      if ((int)is_lsf + (int)is_eps + (int)is_deps > 1) atomicExch(conflict, 1);
    }
  }
}

// The face weights of the lpld operators, eps_0 eps_f / (eps_0 + eps_f)
// for every interior cell and face of a set of boxes (the reference's
// expression; ghost cells read as stored), taken once per call so that the
// sweeps, residuals and restrictions of its cycles do not divide per face and
// cell.
template <int D, int NC>
__global__ void k_coef(BoxSet bs, const long long* __restrict__ offg, const long long* __restrict__ offi,
                       const double* __restrict__ eps, double* __restrict__ coef) {
  using G = Geo<D, NC>;
  const long long total = (long long)bs.n * G::SI * (2 * D);
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(it % (2 * D));
    const long long cell = it / (2 * D);
    const int b = (int)(cell / G::SI), q = (int)(cell % G::SI);
    const int s = bs.lo + b;
    const int i = q % NC + 1, j = (q / NC) % NC + 1, kz = D == 3 ? q / (NC * NC) + 1 : 0;
    const double* e = eps + offg[s];
    const int c = G::g(i, j, kz);
    const double a0 = e[c], a = e[c + nb_off<D, NC>(k)];
    const double p = a0 * a;
    // Equal eps of a moderate size (2^-400 <= |eps| <= 2^500, so eps^2 is a
    // normal number and a non-zero rounding error of it is at least 2^-904,
    // which the fused multiply-add shows) whose square is exact: p / (2 eps)
    // is eps / 2 in exact arithmetic, and the quotient and eps * 0.5 both
    // round it the same way. Other values (0, tiny, huge, non-finite) divide.
    const double ma = fabs(a0);
    const bool exact_half = a0 == a && ma >= 0x1p-400 && ma <= 0x1p500 && fma(a0, a0, -p) == 0.0;
    coef[(offi[s] + q) * (2 * D) + k] = exact_half ? a0 * 0.5 : qdiv(p, a0 + a);
  }
}

// One half-sweep (colour from n) on every box of a level with each box's
// operator: mg$D_box_gsrb_lpl (src/m_aX_mg.f90:718-760), _lpld (:810-859),
// mg2_box_gsrb_clpl / _clpld (:1325-1351, :1410-1443), _lpllsf (:1102-1181).
// One thread per updated cell; ghost cells are read as stored.
template <int D, int NC>
__global__ void k_gsrb(Meta m, Op o, BoxSet bs, double* __restrict__ phi, const double* __restrict__ rhs, int n) {
  using G = Geo<D, NC>;
  constexpr int HALF = G::SI / 2;
  constexpr int NG = NC + 2;
  const long long total = (long long)bs.n * HALF;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(it / HALF), q = (int)(it % HALF);
    const int s = bs.lo + b;
    if (!m.active[m.tree[s]]) continue;
    const int p = q % (NC / 2);
    const int j = (q / (NC / 2)) % NC + 1, k = D == 3 ? q / ((NC / 2) * NC) + 1 : 0;
    const int i0 = 2 - ((n ^ (D == 3 ? k + j : j)) & 1);
    const int i = i0 + 2 * p;
    const SlotDesc& d = m.desc[s];
    double* u = phi + d.offg;
    const int c = G::g(i, j, k);
    const double f = rhs[d.offi + G::in(i, j, D == 3 ? k : 1)];
    const int kind = kind_of(o, s);
    switch (kind) {
      case kLpl:
        if constexpr (D == 2) {
          u[c] = 0.25 * (u[c + 1] + u[c - 1] + u[c + NG] + u[c - NG] - d.dx2 * f);
        } else {
          const double sixth = 1 / 6.0;
          u[c] = sixth * (u[c + 1] + u[c - 1] + u[c + NG] + u[c - NG] + u[c + NG * NG] + u[c - NG * NG] - d.dx2 * f);
        }
        break;
      case kClpl: {
        double r1, r2;
        rfac(i, (o.ix[(size_t)s * D] - 1) * NC, r1, r2);
        u[c] = 0.25 * (r1 * u[c - 1] + r2 * u[c + 1] + u[c + NG] + u[c - NG] - d.dx2 * f);
        break;
      }
      case kLsf: {
        double dd[6], val[6];
        lsf_stencil<D, NC>(u, o.lsf + d.offg, o.bval + d.offg, c, dd, val);
        if constexpr (D == 2) {
          double prod = 1;
          for (int e = 0; e < 4; ++e) prod = prod * dd[e];
          u[c] = qdiv(1, dd[0] * dd[1] + dd[2] * dd[3]) *
                 (qdiv((dd[1] * val[0] + dd[0] * val[1]) * dd[2] * dd[3], dd[0] + dd[1]) +
                  qdiv((dd[3] * val[2] + dd[2] * val[3]) * dd[0] * dd[1], dd[2] + dd[3]) - 0.5 * prod * d.dx2 * f);
        } else {
          u[c] = qdiv(1, qdiv(1, dd[0] * dd[1]) + qdiv(1, dd[2] * dd[3]) + qdiv(1, dd[4] * dd[5])) *
                 (qdiv(dd[1] * val[0] + dd[0] * val[1], (dd[0] + dd[1]) * dd[0] * dd[1]) +
                  qdiv(dd[3] * val[2] + dd[2] * val[3], (dd[2] + dd[3]) * dd[2] * dd[3]) +
                  qdiv(dd[5] * val[4] + dd[4] * val[5], (dd[4] + dd[5]) * dd[4] * dd[5]) - 0.5 * d.dx2 * f);
        }
        break;
      }
      default: {  // kLpld, kClpld
        const bool cyl = kind == kClpld;
        const double* e = o.eps + d.offg;
        const double a0 = e[c];
        double r1 = 1, r2 = 1;
        if (cyl) rfac(i, (o.ix[(size_t)s * D] - 1) * NC, r1, r2);
        // 2 eps_0 eps / (eps_0 + eps) is exactly twice k_coef's weight when
        // both eps lie within 2^-500..2^500 (by their exponents): the product
        // and the quotient are then normal numbers, and a factor 2 commutes
        // with their rounding. Other pairs divide as the reference does.
        auto mid = [](double v) {
          const unsigned ex = (unsigned)((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ffu;
          return ex >= 1023u - 500u && ex <= 1023u + 500u;
        };
        const double* w = (!cyl && o.coef && mid(a0)) ? o.coef + (d.offi + G::in(i, j, D == 3 ? k : 1)) * (2 * D)
                                                       : nullptr;
        double cu = 0.0, cs = 0.0;
#pragma unroll
        for (int kk = 0; kk < 2 * D; ++kk) {
          const int of = nb_off<D, NC>(kk);
          const double a = e[c + of];
          const double ck = (w && mid(a)) ? 2 * w[kk] : qdiv(2 * a0 * a, a0 + a);
          if (cyl) {
            const double rf = kk == 0 ? r1 : kk == 1 ? r2 : 1.0;
            cu = cu + ck * rf * u[c + of];
            cs = cs + ck * rf;
          } else {
            cu = cu + ck * u[c + of];
            cs = cs + ck;
          }
        }
        u[c] = qdiv(cu - d.dx2 * f, cs);
        break;
      }
    }
  }
}

// residual_box (src/m_aX_mg.f90:545-559) with each box's operator:
// tmp = rhs - L phi on the interiors of every box of a set.
template <int D, int NC>
__global__ void k_residual(Meta m, Op o, BoxSet bs, const double* __restrict__ phi, const double* __restrict__ rhs,
                           double* __restrict__ tmp) {
  using G = Geo<D, NC>;
  const long long total = (long long)bs.n * G::SI;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(it / G::SI), q = (int)(it % G::SI);
    const int s = dev::box_at(bs, b);
    if (!m.active[m.tree[s]]) continue;
    const SlotDesc& d = m.desc[s];
    const int i = q % NC + 1, j = (q / NC) % NC + 1, k = D == 3 ? q / (NC * NC) + 1 : 0;
    const int c = G::g(i, j, k);
    const double l = op_at<D, NC>(o, kind_of(o, s), phi, d.offg, s, c, i, d.inv_dx2, d.offi + q);
    tmp[d.offg + c] = rhs[d.offi + q] - l;
  }
}

// One parent cell from the 2^D child cells v (x fastest): the masked average
// of mg$D_box_rstr_lpllsf for level-set children (src/m_aX_mg.f90:1256-1320;
// 1 / n_ch an integer division as there), the weights of a2_restrict_box in
// cylindrical trees (src/m_aX_restrict.f90:90-103), else the plain average
// (Fortran's sum from zero).
template <int D>
__device__ __forceinline__ double restrict_cell(const double* v, bool lsf, const double* lc, double lp, bool cyl,
                                                double w1, double w2) {
  if (lsf) {
    int n_ch = 0;
    double sm = 0.0, sa = 0.0;
    for (int e = 0; e < (1 << D); ++e) {
      sa = sa + v[e];
      if (lp * lc[e] > 0) {
        ++n_ch;
        sm = sm + v[e];
      }
    }
    if (n_ch < (1 << D) && n_ch > 0) return (double)(1 / n_ch) * sm;
    return (D == 2 ? 0.25 : 0.125) * sa;
  }
  if (D == 2 && cyl) {
    double s1 = 0.0, s2 = 0.0;
    s1 = s1 + v[0];
    s1 = s1 + v[2];
    s2 = s2 + v[1];
    s2 = s2 + v[3];
    return 0.25 * (w1 * s1 + w2 * s2);
  }
  double s = 0.0;
  for (int e = 0; e < (1 << D); ++e) s = s + v[e];
  return (D == 2 ? 0.25 : 0.125) * s;
}

// a2_cyl_child_weights (src/m_aX_t.f90:516-528) at index i of the parent
// slot P: the radius of that cell's centre (a2_cyl_radius_cc, :508-514).
template <int D>
__device__ __forceinline__ void cyl_weights(const Op& o, const SlotDesc& dp, int P, int i, double& w1, double& w2) {
  const double r = o.rmin[(size_t)P * D] + (i - 0.5) * dp.dr;
  const double t = 0.25 * dp.dr / r;
  w1 = 1 - t;
  w2 = 1 + t;
}

// The fine side of update_coarse (src/m_aX_mg.f90:441-462) and of
// set_coarse_phi_rhs (:496-503): each child's residual and phi restricted to
// its parent by mg%box_rstr. The residual is computed here per fine cell; with
// store_res it is also left in the child's tmp (set_coarse_phi_rhs),
// otherwise the child's tmp keeps its value (update_coarse restores it).
template <int D, int NC>
__global__ void k_restrict(Meta m, Op o, BoxSet bs, double* __restrict__ phi, const double* __restrict__ rhs,
                           double* __restrict__ tmp, int lvl, int store_res) {
  using G = Geo<D, NC>;
  constexpr int H = NC / 2;
  constexpr int PER = D == 2 ? H * H : H * H * H;
  const int ncp = lvl >= 2 ? NC : H;  // parents of levels <= 1 are half the size
  const int ngp = ncp + 2;
  const long long total = (long long)bs.n * PER;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(it / PER), q = (int)(it % PER);
    const int s = bs.lo + b;
    if (!m.active[m.tree[s]]) continue;
    const SlotDesc& d = m.desc[s];
    const SlotDesc& dp = m.desc[d.parent];
    const int i = q % H + 1, j = (q / H) % H + 1, k = D == 3 ? q / (H * H) + 1 : 1;
    int off[3] = {0, 0, 0};
    if (lvl >= 2)
      for (int e = 0; e < D; ++e) off[e] = ((d.qd >> e) & 1) * H;
    const int kind = kind_of(o, s);
    double r[8], p[8], lc[8];
    int e = 0;
#pragma unroll
    for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii, ++e) {
          const int fi = 2 * i - 1 + ii, fj = 2 * j - 1 + jj, fk = D == 3 ? 2 * k - 1 + kk : 0;
          const int c = G::g(fi, fj, fk);
          const long long qf = d.offi + G::in(fi, fj, D == 3 ? fk : 1);
          r[e] = rhs[qf] - op_at<D, NC>(o, kind, phi, d.offg, s, c, fi, d.inv_dx2, qf);
          if (store_res) tmp[d.offg + c] = r[e];
          p[e] = phi[d.offg + c];
          lc[e] = kind == kLsf ? o.lsf[d.offg + c] : 0.0;
        }
    const long long pc =
        (long long)(off[0] + i) + (long long)ngp * ((off[1] + j) + (D == 3 ? (long long)ngp * (off[2] + k) : 0));
    const double lp = kind == kLsf ? o.lsf[dp.offg + pc] : 0.0;
    double w1 = 1, w2 = 1;
    if (o.cyl) cyl_weights<D>(o, dp, d.parent, i, w1, w2);
    tmp[dp.offg + pc] = restrict_cell<D>(r, kind == kLsf, lc, lp, o.cyl, w1, w2);
    phi[dp.offg + pc] = restrict_cell<D>(p, kind == kLsf, lc, lp, o.cyl, w1, w2);
  }
}

// init_phi_rhs (src/m_aX_mg.f90:520-543) on one level: each child's rhs
// restricted to its parent by mg%box_rstr (phi is cleared separately).
template <int D, int NC>
__global__ void k_init_level(Meta m, Op o, BoxSet bs, double* __restrict__ rhs, int lvl) {
  using G = Geo<D, NC>;
  constexpr int H = NC / 2;
  constexpr int PER = D == 2 ? H * H : H * H * H;
  const int ncp = lvl >= 2 ? NC : H;
  const long long total = (long long)bs.n * PER;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(it / PER), q = (int)(it % PER);
    const int s = bs.lo + b;
    if (!m.active[m.tree[s]]) continue;
    const SlotDesc& d = m.desc[s];
    const SlotDesc& dp = m.desc[d.parent];
    const int i = q % H + 1, j = (q / H) % H + 1, k = D == 3 ? q / (H * H) + 1 : 1;
    int off[3] = {0, 0, 0};
    if (lvl >= 2)
      for (int e = 0; e < D; ++e) off[e] = ((d.qd >> e) & 1) * H;
    const int kind = kind_of(o, s);
    double v[8], lc[8];
    int e = 0;
#pragma unroll
    for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii, ++e) {
          const int fi = 2 * i - 1 + ii, fj = 2 * j - 1 + jj, fk = D == 3 ? 2 * k - 1 + kk : 0;
          v[e] = rhs[d.offi + G::in(fi, fj, D == 3 ? fk : 1)];
          lc[e] = kind == kLsf ? o.lsf[d.offg + G::g(fi, fj, fk)] : 0.0;
        }
    const int pi = off[0] + i, pj = off[1] + j, pk = D == 3 ? off[2] + k : 1;
    const long long pc = (long long)(pi - 1) + (long long)ncp * ((pj - 1) + (D == 3 ? (long long)ncp * (pk - 1) : 0));
    const int ngp = ncp + 2;
    const double lp =
        kind == kLsf ? o.lsf[dp.offg + pi + (long long)ngp * (pj + (D == 3 ? (long long)ngp * pk : 0))] : 0.0;
    double w1 = 1, w2 = 1;
    if (o.cyl) cyl_weights<D>(o, dp, d.parent, i, w1, w2);
    rhs[dp.offi + pc] = restrict_cell<D>(v, kind == kLsf, lc, lp, o.cyl, w1, w2);
  }
}

// The coarse side of update_coarse (src/m_aX_mg.f90:468-479): on each parent
// rhs = L phi + tmp, then (copy_tmp) tmp = phi over the whole box.
template <int D, int NC>
__global__ void k_coarse(Meta m, Op o, BoxSet bs, const double* __restrict__ phi, double* __restrict__ rhs,
                         double* __restrict__ tmp, int copy_tmp) {
  using G = Geo<D, NC>;
  const long long total = (long long)bs.n * G::SG;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(it / G::SG), c = (int)(it % G::SG);
    const int s = dev::box_at(bs, b);
    if (!m.active[m.tree[s]]) continue;
    const SlotDesc& d = m.desc[s];
    const int i = c % (NC + 2), j = (c / (NC + 2)) % (NC + 2), k = D == 3 ? c / ((NC + 2) * (NC + 2)) : 1;
    const bool inner = i >= 1 && i <= NC && j >= 1 && j <= NC && k >= 1 && k <= NC;
    if (inner) {
      const long long qi = d.offi + G::in(i, j, D == 3 ? k : 1);
      const double l = op_at<D, NC>(o, kind_of(o, s), phi, d.offg, s, c, i, d.inv_dx2, qi);
      rhs[qi] = l + tmp[d.offg + c];
    }
    if (copy_tmp) tmp[d.offg + c] = phi[d.offg + c];
  }
}

// correct_children, first part (src/m_aX_mg.f90:380-386): tmp = phi - tmp
// on the whole parent box.
template <int D, int NC>
__global__ void k_tmp_diff(Meta m, BoxSet bs, const double* __restrict__ phi, double* __restrict__ tmp) {
  using G = Geo<D, NC>;
  const long long total = (long long)bs.n * G::SG;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int s = dev::box_at(bs, (int)(it / G::SG));
    if (!m.active[m.tree[s]]) continue;
    const long long o = m.offg[s] + it % G::SG;
    tmp[o] = phi[o] - tmp[o];
  }
}

// correct_children, second part: each child's correction from its parent's
// tmp by mg%box_corr (the child's operator in auto mode): a$D_prolong2 with
// add for (c)lpl (src/m_aX_prolong.f90:243-348), mg$D_box_corr_lpld for
// (c)lpld (src/m_aX_mg.f90:907-985), mg$D_box_corr_lpllsf (:1021-1099). One
// thread per child cell; parents on levels <= 0 have one child of twice their
// size.
template <int D, int NCC>
__global__ void k_correct(Meta m, Op o, BoxSet parents, int nch, double* __restrict__ phi,
                          const double* __restrict__ tmp, int lvl_child) {
  using G = Geo<D, NCC>;
  constexpr int H = NCC / 2;
  const int ncp = lvl_child >= 2 ? NCC : H;
  const int ngp = ncp + 2;
  const long long total = (long long)parents.n * nch * G::SI;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % G::SI);
    const int ch = (int)((it / G::SI) % nch);
    const int P = dev::box_at(parents, (int)(it / G::SI / nch));
    if (!m.active[m.tree[P]]) continue;
    const int C = m.first_child[P] + ch;
    const SlotDesc& dc = m.desc[C];
    const SlotDesc& dp = m.desc[P];
    const int i = q % NCC + 1, j = (q / NCC) % NCC + 1, k = D == 3 ? q / (NCC * NCC) + 1 : 0;
    int off[3] = {0, 0, 0};
    if (lvl_child >= 2)
      for (int e = 0; e < D; ++e) off[e] = ((dc.qd >> e) & 1) * H;
    const int x[3] = {i, j, k};
    int c1[3] = {0, 0, 0}, c2[3] = {0, 0, 0};
    for (int e = 0; e < D; ++e) {
      c1[e] = off[e] + ((x[e] + 1) >> 1);
      c2[e] = c1[e] + 1 - 2 * (x[e] & 1);
    }
    auto P_ = [&](const double* v, int a, int b_, int c_) {
      return v[dp.offg + a + (long long)ngp * (b_ + (D == 3 ? (long long)ngp * c_ : 0))];
    };
    double& out = phi[dc.offg + G::g(i, j, k)];
    const int kind = kind_of(o, C);
    if (kind == kLpl || kind == kClpl) {
      // a$D_prolong2: f0 +- fx +- fy (+- fz) + second differences, minus at
      // odd fine indices
      const int ic = c1[0], jc = c1[1], kc = c1[2];
      const double f0 = P_(tmp, ic, jc, kc);
      const double fx = 0.125 * (P_(tmp, ic + 1, jc, kc) - P_(tmp, ic - 1, jc, kc));
      const double fy = 0.125 * (P_(tmp, ic, jc + 1, kc) - P_(tmp, ic, jc - 1, kc));
      const double fxx = 0.03125 * (P_(tmp, ic - 1, jc, kc) - 2 * f0 + P_(tmp, ic + 1, jc, kc));
      const double fyy = 0.03125 * (P_(tmp, ic, jc - 1, kc) - 2 * f0 + P_(tmp, ic, jc + 1, kc));
      double v = (i & 1) ? f0 - fx : f0 + fx;
      v = (j & 1) ? v - fy : v + fy;
      if constexpr (D == 2) {
        out = v + (fxx + fyy) + out;
      } else {
        const double fz = 0.125 * (P_(tmp, ic, jc, kc + 1) - P_(tmp, ic, jc, kc - 1));
        const double fzz = 0.03125 * (P_(tmp, ic, jc, kc - 1) - 2 * f0 + P_(tmp, ic, jc, kc + 1));
        v = (k & 1) ? v - fz : v + fz;
        out = v + (fxx + fyy + fzz) + out;
      }
    } else if (kind == kLsf) {
      // the fine cell's level set against the 1 + D coarse points; the
      // correction is 0 at the interface
      const double la = o.lsf[dc.offg + G::g(i, j, k)];
      double dist[4], val[4];
      for (int e = 0; e <= D; ++e) {
        int cc[3] = {c1[0], c1[1], c1[2]};
        if (e > 0) cc[e - 1] = c2[e - 1];
        lsf_dist_val(la, 0.0, P_(o.lsf, cc[0], cc[1], cc[2]), P_(tmp, cc[0], cc[1], cc[2]), 0.0, dist[e], val[e]);
      }
      double cw[4];
      if constexpr (D == 2) {
        cw[0] = 2 * dist[1] * dist[2];
        cw[1] = dist[0] * dist[2];
        cw[2] = dist[0] * dist[1];
      } else {
        cw[0] = dist[1] * dist[2] * dist[3];
        cw[1] = dist[0] * dist[2] * dist[3];
        cw[2] = dist[0] * dist[1] * dist[3];
        cw[3] = dist[0] * dist[1] * dist[2];
      }
      double s1 = 0.0, s2 = 0.0;
      for (int e = 0; e <= D; ++e) s1 = s1 + cw[e] * val[e];
      for (int e = 0; e <= D; ++e) s2 = s2 + cw[e];
      out = out + qdiv(s1, s2);
    } else {
      const double u0 = P_(tmp, c1[0], c1[1], c1[2]);
      const double a0 = P_(o.eps, c1[0], c1[1], c1[2]);
      double sm = 0.0;
#pragma unroll
      for (int e = 0; e < D; ++e) {
        int cc[3] = {c1[0], c1[1], c1[2]};
        cc[e] = c2[e];
        const double u = P_(tmp, cc[0], cc[1], cc[2]);
        const double a = P_(o.eps, cc[0], cc[1], cc[2]);
        if constexpr (D == 2)
          sm = sm + qdiv(a0 * u0 + a * u, a0 + a);
        else
          sm = sm + qdiv(a0 * u0 + a * (1.5 * u - 0.5 * u0), a0 + a);
      }
      out = out + (D == 2 ? 0.5 : 1 / 3.0) * sm;
    }
  }
}

}  // namespace opdev

namespace {

template <int N> using IC = std::integral_constant<int, N>;

template <class F>
bool with_nc_op(int D, int nc, F&& f) {
  if (D == 2) {
    switch (nc) {
      case 2: f(IC<2>{}, IC<2>{}); return true;
      case 4: f(IC<2>{}, IC<4>{}); return true;
      case 8: f(IC<2>{}, IC<8>{}); return true;
      case 16: f(IC<2>{}, IC<16>{}); return true;
    }
  } else {
    switch (nc) {
      case 2: f(IC<3>{}, IC<2>{}); return true;
      case 4: f(IC<3>{}, IC<4>{}); return true;
      case 8: f(IC<3>{}, IC<8>{}); return true;
    }
  }
  return false;
}

int grid_n(long long items, int n_sm) {
  return (int)std::max(1LL, std::min((items + 255) / 256, (long long)n_sm * 16));
}

dev::Meta meta_for(const DevMeta& d) {
  dev::Meta m;
  m.tree = d.tree;
  m.parent = d.parent;
  m.first_child = d.first_child;
  m.offg = d.offg;
  m.offi = d.offi;
  m.bcval = d.bcval;
  m.active = d.active;
  m.desc = d.desc;
  m.nbo2 = d.nbo2;
  m.err = d.err;
  m.wait_limit = d.wait_limit;
  return m;
}

}  // namespace

const double* Forest::eps_ptr() const { return i_eps >= 0 ? var_ptr(i_eps) : d64.phi; }

opdev::Op Forest::op_args() const {
  opdev::Op o;
  o.op = op;
  o.cyl = plan.cyl;
  o.tags = d_tags;
  o.eps = eps_ptr();
  o.lsf = i_lsf >= 0 ? var_ptr(i_lsf) : d64.phi;
  o.bval = i_bval >= 0 ? var_ptr(i_bval) : d64.phi;
  o.ix = d_ix;
  o.rmin = meta.rmin;
  o.coef = (i_eps >= 0 && d_coef && (op == AFV_OP_LPLD || op == AFV_OP_AUTO)) ? d_coef : nullptr;
  return o;
}

// mg$D_init_mg's checks (src/m_aX_mg.f90:130-154) and the choice of
// mg%box_op / box_gsrb / box_corr / box_rstr. For AFV_OP_AUTO the tags of
// mg$D_set_box_tag are taken here from the current eps and level set (ghost
// cells included), where the reference takes each box's tag at first use.
int Forest::set_operator(int new_op, int new_i_eps, int new_i_lsf, int new_i_bval, std::string& err) {
  switch (new_op) {
    case AFV_OP_LPL: case AFV_OP_LPLD: case AFV_OP_AUTO: case AFV_OP_CLPL: case AFV_OP_CLPLD: case AFV_OP_LPLLSF:
      break;
    default:
      return err = "unknown operator", AFV_ERR_INVALID;
  }
  if ((new_op == AFV_OP_CLPL || new_op == AFV_OP_CLPLD) && !plan.cyl)
    return err = "the cylindrical operators need cylindrical trees (afv_tree_set_coord)", AFV_ERR_INVALID;
  auto is_var = [&](int iv) { return iv >= 3 && iv < n_cc_vars() && var_ptr(iv); };
  const bool need_eps = new_op == AFV_OP_LPLD || new_op == AFV_OP_CLPLD;
  if (need_eps && !is_var(new_i_eps))
    return err = "eps must be an extra cell variable (afv_forest_add_vars)", AFV_ERR_INVALID;
  if ((new_i_lsf >= 0) != (new_i_bval >= 0)) return err = "you have to set both i_lsf and i_bval", AFV_ERR_INVALID;
  if (new_op == AFV_OP_LPLLSF && new_i_lsf < 0) return err = "lpllsf needs i_lsf and i_bval", AFV_ERR_INVALID;
  if (new_i_lsf >= 0 && (!is_var(new_i_lsf) || !is_var(new_i_bval)))
    return err = "lsf and bval must be extra cell variables (afv_forest_add_vars)", AFV_ERR_INVALID;
  if (new_op == AFV_OP_AUTO && new_i_eps >= 0 && !is_var(new_i_eps))
    return err = "eps must be an extra cell variable (afv_forest_add_vars)", AFV_ERR_INVALID;
  drop_graphs();
  if (!d_tags) {
    if (cudaMallocAsync((void**)&d_tags, sizeof(int) * std::max(1, plan.n_slots), stream) != cudaSuccess)
      return err = "device allocation failed", AFV_ERR_NOMEM;
    bytes += sizeof(int) * plan.n_slots;
  }
  if (plan.cyl && !d_ix) {
    const size_t n = (size_t)std::max(1, plan.n_slots) * plan.dim;
    if (cudaMallocAsync((void**)&d_ix, sizeof(int) * n, stream) != cudaSuccess)
      return err = "device allocation failed", AFV_ERR_NOMEM;
    bytes += sizeof(int) * n;
    if (!plan.ix.empty() &&
        cudaMemcpyAsync(d_ix, plan.ix.data(), sizeof(int) * plan.ix.size(), cudaMemcpyHostToDevice, stream) !=
            cudaSuccess)
      return err = "set_operator: CUDA error", AFV_ERR_CUDA;
  }
  const int t_eps = (need_eps || new_op == AFV_OP_AUTO) ? new_i_eps : -1;
  const int t_lsf = (new_op == AFV_OP_LPLLSF || new_op == AFV_OP_AUTO) ? new_i_lsf : -1;
  int* conflict = nullptr;
  if (new_op == AFV_OP_AUTO) {
    if (cudaMallocAsync((void**)&conflict, sizeof(int), stream) != cudaSuccess)
      return err = "device allocation failed", AFV_ERR_NOMEM;
    cudaMemsetAsync(conflict, 0, sizeof(int), stream);
    for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
      const int nbx = lvl_n(l);
      if (!nbx) continue;
      with_nc_op(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
        constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
        opdev::k_tags<D, NC><<<grid_n(32LL * nbx, n_sm), 256, 0, stream>>>(
            level_set(l), meta.offg, t_eps >= 0 ? var_ptr(t_eps) : nullptr, t_lsf >= 0 ? var_ptr(t_lsf) : nullptr,
            d_tags, conflict);
        ++n_launches;
      });
    }
  }
  if (t_eps >= 0 && !d_coef) {  // room for the lpld face weights (gen_coef)
    const size_t n = (size_t)std::max(1LL, plan.n_elem_i) * 2 * plan.dim;
    if (cudaMallocAsync((void**)&d_coef, sizeof(double) * n, stream) != cudaSuccess)
      return err = "device allocation failed", AFV_ERR_NOMEM;
    bytes += sizeof(double) * n;
  }
  int h_conflict = 0;
  if (conflict) {
    cudaMemcpyAsync(&h_conflict, conflict, sizeof(int), cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(conflict, stream);
  }
  if (cudaStreamSynchronize(stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return err = "set_operator: CUDA error", AFV_ERR_CUDA;
  if (h_conflict) return err = "a box has both a level set crossing and a (variable) eps", AFV_ERR_INVALID;
  op = new_op;
  i_eps = t_eps;
  i_lsf = t_lsf;
  i_bval = t_lsf >= 0 ? new_i_bval : -1;
  return AFV_OK;
}

// The lpld face weights from the current eps, on every level, enqueued at
// the start of each FP64 routine (and in each solve's graph) so that a call
// sees eps as it is when the call runs, as the reference's operators that
// read eps at every use.
void Forest::gen_coef() {
  if (i_eps < 0 || !d_coef || (op != AFV_OP_LPLD && op != AFV_OP_AUTO)) return;
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
    const int nbx = lvl_n(l);
    if (!nbx) continue;
    with_nc_op(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      opdev::k_coef<D, NC><<<grid_n((long long)nbx * G::SI * 2 * D, n_sm), 256, 0, stream>>>(
          level_set(l), meta.offg, meta.offi, var_ptr(i_eps), d_coef);
      ++n_launches;
    });
  }
}

// gsrb_boxes (src/m_aX_mg.f90:397-420): each half-sweep, then the level's
// ghost fill.
void Forest::gen_gsrb_boxes(int lvl, int n_cycle) {
  const int nbx = lvl_n(lvl);
  if (!nbx || n_cycle <= 0) return;
  const dev::Meta m = meta_for(meta);
  const opdev::Op o = op_args();
  for (int n = 1; n <= 2 * n_cycle; ++n) {
    with_nc_op(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      opdev::k_gsrb<D, NC><<<grid_n((long long)nbx * G::SI / 2, n_sm), 256, 0, stream>>>(m, o, level_set(lvl), d64.phi,
                                                                                          d64.rhs, n);
      ++n_launches;
    });
    fill64(lvl);
  }
}

// update_coarse (copy_tmp) and set_coarse_phi_rhs (without), src/m_aX_mg.f90:424-517.
void Forest::gen_update_coarse(int lvl, bool copy_tmp) {
  const int nbx = lvl_n(lvl);
  if (!nbx || lvl <= plan.min_lvl) return;
  const dev::Meta m = meta_for(meta);
  const opdev::Op o = op_args();
  with_nc_op(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_restrict<D, NC><<<grid_n((long long)nbx * G::SI / (1 << D), n_sm), 256, 0, stream>>>(
        m, o, level_set(lvl), d64.phi, d64.rhs, d64.tmp, lvl, copy_tmp ? 0 : 1);
    ++n_launches;
  });
  fill64(lvl - 1);
  const int np = n_parents(lvl - 1);
  if (!np) return;
  with_nc_op(plan.dim, plan.nc_at(lvl - 1), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_coarse<D, NC><<<grid_n((long long)np * G::SG, n_sm), 256, 0, stream>>>(
        m, o, dev::BoxSet{parents_list(lvl - 1), 0, np, 0, 0}, d64.phi, d64.rhs, d64.tmp, copy_tmp ? 1 : 0);
    ++n_launches;
  });
}

// init_phi_rhs (src/m_aX_mg.f90:520-543): phi cleared on the levels above
// the lowest and rhs restricted downwards, level by level, by mg%box_rstr.
void Forest::gen_init_phi_rhs() {
  const dev::Meta m = meta_for(meta);
  const opdev::Op o = op_args();
  for (int l = plan.max_lvl; l >= plan.min_lvl + 1; --l) {
    const int nbx = lvl_n(l);
    if (!nbx) continue;
    with_nc_op(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      constexpr int VW = dev::Vec<double>::w;
      dev::k_box_op<D, NC, double><<<grid_n((long long)nbx * (G::SG / VW), n_sm), 256, 0, stream>>>(
          m, level_set(l), d64.phi, nullptr, 0);
      opdev::k_init_level<D, NC><<<grid_n((long long)nbx * G::SI / (1 << D), n_sm), 256, 0, stream>>>(
          m, o, level_set(l), d64.rhs, l);
      n_launches += 2;
    });
  }
}

// correct_children on the parents of level lp (src/m_aX_mg.f90:368-395).
void Forest::gen_correct(int lp) {
  const int np = n_parents(lp);
  if (!np) return;
  const dev::Meta m = meta_for(meta);
  const opdev::Op o = op_args();
  const dev::BoxSet pb{parents_list(lp), 0, np, 0, 0};
  with_nc_op(plan.dim, plan.nc_at(lp), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_tmp_diff<D, NC><<<grid_n((long long)np * G::SG, n_sm), 256, 0, stream>>>(m, pb, d64.phi, d64.tmp);
    ++n_launches;
  });
  const int nch = lp >= 1 ? (1 << plan.dim) : 1;
  with_nc_op(plan.dim, plan.nc_at(lp + 1), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_correct<D, NC><<<grid_n((long long)np * nch * G::SI, n_sm), 256, 0, stream>>>(m, o, pb, nch, d64.phi,
                                                                                            d64.tmp, lp + 1);
    ++n_launches;
  });
}

// residual_box on every box of a level; with norm, max |tmp| over the leaves
// per tree into the striped norms.
void Forest::gen_residual(int lvl, unsigned long long* norm) {
  const int nbx = lvl_n(lvl);
  if (!nbx) return;
  const dev::Meta m = meta_for(meta);
  const opdev::Op o = op_args();
  with_nc_op(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_residual<D, NC><<<grid_n((long long)nbx * G::SI, n_sm), 256, 0, stream>>>(m, o, level_set(lvl), d64.phi,
                                                                                       d64.rhs, d64.tmp);
    ++n_launches;
    const int nl = n_leaves(lvl);
    if (norm && nl) {
      constexpr int PER_BOX = G::SI < 32 ? G::SI : 32;
      constexpr int BPC = dev::kThreads / PER_BOX;
      dev::k_maxabs<D, NC, double><<<grid_n((long long)(nl + BPC - 1) / BPC * 256, n_sm), dev::kThreads, 0, stream>>>(
          m, dev::BoxSet{leaves_list(lvl), 0, nl, 0, 0}, (const double*)d64.tmp, 1, norm);
      ++n_launches;
    }
  });
}

// mg$D_fas_vcycle (src/m_aX_mg.f90:208-255) with the forest's operator.
void Forest::gen_vcycle(const MgOpts& mg, int highest, bool set_residual) {
  const int l0 = plan.min_lvl;
  for (int l = highest; l >= l0 + 1; --l) {
    gen_gsrb_boxes(l, mg.n_down);
    gen_update_coarse(l, true);
  }
  gen_gsrb_boxes(l0, mg.n_base);
  for (int l = l0 + 1; l <= highest; ++l) {
    gen_correct(l - 1);
    fill64(l);
    gen_gsrb_boxes(l, mg.n_up);
  }
  if (set_residual)
    for (int l = l0; l <= highest; ++l) gen_residual(l, nullptr);
}

}  // namespace afv
