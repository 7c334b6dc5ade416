// Operator variants behind the same FAS V-cycle (FP64): the variable-
// coefficient Laplacian div(eps grad phi) of mg$D_box_gsrb_lpld,
// mg$D_box_lpld and mg$D_box_corr_lpld (src/m_aX_mg.f90:810-985), and the
// per-box dispatch of mg$D_auto_gsrb / _op / _corr with the tags of
// mg$D_set_box_tag (src/m_aX_mg.f90:562-706): boxes whose eps is 1 everywhere
// take the constant-coefficient operators, the others the lpld ones.
//
// The schedule is the reference's, operator by operator: every half-sweep is
// followed by a ghost fill of its level (gsrb_boxes, src/m_aX_mg.f90:
// 397-420), update_coarse restricts the residual and phi (:424-480), and
// correct_children forms tmp = phi - tmp on the parents before the children
// take their correction (:368-395). Each kernel takes one thread per updated
// cell and keeps the reference's expression order, so results are
// bit-identical to the reference's routines (-fmad=false). The constant-
// coefficient solver keeps its own fused kernels (solver.cu); this path is
// taken only when a forest's operator is not the plain Laplacian.
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

enum { kTagNormal = 1, kTagCeps = 3, kTagVeps = 4 };  // mg_normal_box, mg_ceps_box, mg_veps_box

__device__ __forceinline__ bool is_lpld(int op, const int* __restrict__ tags, int s) {
  return op == AFV_OP_LPLD || (op == AFV_OP_AUTO && tags[s] != kTagNormal);
}

// Offsets of the 2D face neighbours of a cell in a ghosted box, in the
// reference's order: (i-1), (i+1), (j-1), (j+1)[, (k-1), (k+1)].
template <int D, int NC>
__device__ __forceinline__ int nb_off(int k) {
  constexpr int NG = NC + 2;
  const int step = k < 2 ? 1 : (k < 4 ? NG : NG * NG);
  return (k & 1) ? step : -step;
}

// L phi at ghosted index c: mg$D_box_lpl (src/m_aX_mg.f90:763-797) or
// mg$D_box_lpld (:861-905).
template <int D, int NC>
__device__ __forceinline__ double op_at(const double* __restrict__ u, const double* __restrict__ e, int c,
                                        double inv_dr_sq, bool lpld) {
  if (!lpld) {
    if constexpr (D == 2)
      return inv_dr_sq * (u[c - 1] + u[c + 1] + u[c - (NC + 2)] + u[c + (NC + 2)] - 4 * u[c]);
    else
      return inv_dr_sq * (u[c - 1] + u[c + 1] + u[c - (NC + 2)] + u[c + (NC + 2)] +
                          u[c - (NC + 2) * (NC + 2)] + u[c + (NC + 2) * (NC + 2)] - 6 * u[c]);
  }
  const double u0 = u[c], a0 = e[c];
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 2 * D; ++k) {
    const int o = nb_off<D, NC>(k);
    const double a = e[c + o];
    s = s + a0 * a / (a0 + a) * (u[c + o] - u0);
  }
  return inv_dr_sq * 2 * s;
}

// mg$D_set_box_tag (src/m_aX_mg.f90:672-706) without the level-set part:
// min and max of eps over the whole box, ghost cells included.
template <int D, int NC>
__global__ void k_tags(BoxSet bs, const long long* __restrict__ offg, const double* __restrict__ eps,
                       int* __restrict__ tags) {
  using G = Geo<D, NC>;
  const int lane = threadIdx.x & 31;
  const int warps = (int)(gridDim.x * blockDim.x) >> 5;
  for (int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < bs.n; b += warps) {
    const int s = bs.lo + b;
    const double* e = eps + offg[s];
    double mn = e[0], mx = e[0];
    for (int q = lane; q < G::SG; q += 32) {
      mn = fmin(mn, e[q]);
      mx = fmax(mx, e[q]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
      const bool deps = mx > mn;
      const bool ceps = !deps && (mn < 1 || mn > 1);
      tags[s] = deps ? kTagVeps : ceps ? kTagCeps : kTagNormal;
    }
  }
}

// One half-sweep (colour from n) on every box of a level: mg$D_box_gsrb_lpl
// (src/m_aX_mg.f90:718-760) or mg$D_box_gsrb_lpld (:810-859). One thread per
// updated cell; ghost cells are read as stored.
template <int D, int NC>
__global__ void k_gsrb(Meta m, BoxSet bs, double* __restrict__ phi, const double* __restrict__ rhs,
                       const double* __restrict__ eps, const int* __restrict__ tags, int op, int n) {
  using G = Geo<D, NC>;
  constexpr int HALF = G::SI / 2;
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
    if (!is_lpld(op, tags, s)) {
      if constexpr (D == 2) {
        u[c] = 0.25 * (u[c + 1] + u[c - 1] + u[c + (NC + 2)] + u[c - (NC + 2)] - d.dx2 * f);
      } else {
        const double sixth = 1 / 6.0;
        constexpr int OZ = (NC + 2) * (NC + 2);
        u[c] = sixth * (u[c + 1] + u[c - 1] + u[c + (NC + 2)] + u[c - (NC + 2)] + u[c + OZ] + u[c - OZ] -
                        d.dx2 * f);
      }
    } else {
      const double* e = eps + d.offg;
      const double a0 = e[c];
      double cu = 0.0, cs = 0.0;
#pragma unroll
      for (int kk = 0; kk < 2 * D; ++kk) {
        const int o = nb_off<D, NC>(kk);
        const double a = e[c + o];
        const double ck = 2 * a0 * a / (a0 + a);
        cu = cu + ck * u[c + o];
        cs = cs + ck;
      }
      u[c] = (cu - d.dx2 * f) / cs;
    }
  }
}

// residual_box (src/m_aX_mg.f90:545-559) with the forest's operator:
// tmp = rhs - L phi on the interiors of every box of a set.
template <int D, int NC>
__global__ void k_residual(Meta m, BoxSet bs, const double* __restrict__ phi, const double* __restrict__ rhs,
                           double* __restrict__ tmp, const double* __restrict__ eps, const int* __restrict__ tags,
                           int op) {
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
    const double l = op_at<D, NC>(phi + d.offg, eps + d.offg, c, d.inv_dx2, is_lpld(op, tags, s));
    tmp[d.offg + c] = rhs[d.offi + q] - l;
  }
}

// The fine side of update_coarse (src/m_aX_mg.f90:441-462) and of
// set_coarse_phi_rhs (:496-503): each child's residual and phi restricted to
// its parent (mg$D_box_rstr_lpl = a$D_restrict_box, the Fortran sum from
// zero). The residual is computed here per fine cell; with store_res it is
// also left in the child's tmp (set_coarse_phi_rhs), otherwise the child's
// tmp keeps its value (update_coarse restores it).
template <int D, int NC>
__global__ void k_restrict(Meta m, BoxSet bs, double* __restrict__ phi, const double* __restrict__ rhs,
                           double* __restrict__ tmp, const double* __restrict__ eps, const int* __restrict__ tags,
                           int op, int lvl, int store_res) {
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
    const bool lpld = is_lpld(op, tags, s);
    double sr = 0.0, sp = 0.0;
#pragma unroll
    for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii) {
          const int fi = 2 * i - 1 + ii, fj = 2 * j - 1 + jj, fk = D == 3 ? 2 * k - 1 + kk : 0;
          const int c = G::g(fi, fj, fk);
          const double r = rhs[d.offi + G::in(fi, fj, D == 3 ? fk : 1)] -
                           op_at<D, NC>(phi + d.offg, eps + d.offg, c, d.inv_dx2, lpld);
          if (store_res) tmp[d.offg + c] = r;
          sr = sr + r;
          sp = sp + phi[d.offg + c];
        }
    const double w = D == 2 ? 0.25 : 0.125;
    const long long pc = (long long)(off[0] + i) + (long long)ngp * ((off[1] + j) + (D == 3 ? (long long)ngp * (off[2] + k) : 0));
    tmp[dp.offg + pc] = w * sr;
    phi[dp.offg + pc] = w * sp;
  }
}

// The coarse side of update_coarse (src/m_aX_mg.f90:468-479): on each parent
// rhs = L phi + tmp, then (copy_tmp) tmp = phi over the whole box.
template <int D, int NC>
__global__ void k_coarse(Meta m, BoxSet bs, const double* __restrict__ phi, double* __restrict__ rhs,
                         double* __restrict__ tmp, const double* __restrict__ eps, const int* __restrict__ tags,
                         int op, int copy_tmp) {
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
      const double l = op_at<D, NC>(phi + d.offg, eps + d.offg, c, d.inv_dx2, is_lpld(op, tags, s));
      rhs[d.offi + G::in(i, j, D == 3 ? k : 1)] = l + tmp[d.offg + c];
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
// tmp, by mg$D_box_corr_lpl (a$D_prolong2 with add, src/m_aX_prolong.f90:
// 243-348) or mg$D_box_corr_lpld (src/m_aX_mg.f90:907-985), the child's tag
// choosing in auto mode. One thread per child cell. NCC is the children's
// box size; parents on levels <= 0 have one child of twice their size.
template <int D, int NCC>
__global__ void k_correct(Meta m, BoxSet parents, int nch, double* __restrict__ phi, const double* __restrict__ tmp,
                          const double* __restrict__ eps, const int* __restrict__ tags, int op, int lvl_child) {
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
    double& o = phi[dc.offg + G::g(i, j, k)];
    if (!is_lpld(op, tags, C)) {
      // a$D_prolong2: f0 +- fx +- fy (+- fz) + f2, minus at odd fine indices
      const int ic = c1[0], jc = c1[1], kc = c1[2];
      const double f0 = P_(tmp, ic, jc, kc);
      const double fx = 0.125 * (P_(tmp, ic + 1, jc, kc) - P_(tmp, ic - 1, jc, kc));
      const double fy = 0.125 * (P_(tmp, ic, jc + 1, kc) - P_(tmp, ic, jc - 1, kc));
      const double fxx = 0.03125 * (P_(tmp, ic - 1, jc, kc) - 2 * f0 + P_(tmp, ic + 1, jc, kc));
      const double fyy = 0.03125 * (P_(tmp, ic, jc - 1, kc) - 2 * f0 + P_(tmp, ic, jc + 1, kc));
      double v = (i & 1) ? f0 - fx : f0 + fx;
      v = (j & 1) ? v - fy : v + fy;
      if constexpr (D == 2) {
        o = v + (fxx + fyy) + o;
      } else {
        const double fz = 0.125 * (P_(tmp, ic, jc, kc + 1) - P_(tmp, ic, jc, kc - 1));
        const double fzz = 0.03125 * (P_(tmp, ic, jc, kc - 1) - 2 * f0 + P_(tmp, ic, jc, kc + 1));
        v = (k & 1) ? v - fz : v + fz;
        o = v + (fxx + fyy + fzz) + o;
      }
    } else {
      const double u0 = P_(tmp, c1[0], c1[1], c1[2]);
      const double a0 = P_(eps, c1[0], c1[1], c1[2]);
      double s = 0.0;
#pragma unroll
      for (int e = 0; e < D; ++e) {
        int cc[3] = {c1[0], c1[1], c1[2]};
        cc[e] = c2[e];
        const double u = P_(tmp, cc[0], cc[1], cc[2]);
        const double a = P_(eps, cc[0], cc[1], cc[2]);
        if constexpr (D == 2)
          s = s + (a0 * u0 + a * u) / (a0 + a);
        else
          s = s + (a0 * u0 + a * (1.5 * u - 0.5 * u0)) / (a0 + a);
      }
      o = o + (D == 2 ? 0.5 : 1 / 3.0) * s;
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

int Forest::set_operator(int new_op, int new_i_eps, std::string& err) {
  if (new_op != AFV_OP_LPL && new_op != AFV_OP_LPLD && new_op != AFV_OP_AUTO)
    return err = "unknown operator", AFV_ERR_INVALID;
  if (new_op != AFV_OP_LPL && (new_i_eps < 3 || !var_ptr(new_i_eps)))
    return err = "eps must be an extra cell variable (afv_forest_add_vars)", AFV_ERR_INVALID;
  op = new_op;
  i_eps = new_op == AFV_OP_LPL ? -1 : new_i_eps;
  drop_graphs();
  if (!d_tags) {
    if (cudaMallocAsync((void**)&d_tags, sizeof(int) * std::max(1, plan.n_slots), stream) != cudaSuccess)
      return err = "device allocation failed", AFV_ERR_NOMEM;
    bytes += sizeof(int) * plan.n_slots;
  }
  if (op == AFV_OP_AUTO) {
    for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
      const int nbx = lvl_n(l);
      if (!nbx) continue;
      with_nc_op(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
        constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
        opdev::k_tags<D, NC><<<grid_n(32LL * nbx, n_sm), 256, 0, stream>>>(level_set(l), meta.offg, eps_ptr(),
                                                                         d_tags);
        ++n_launches;
      });
    }
  }
  if (cudaStreamSynchronize(stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return err = "set_operator: CUDA error", AFV_ERR_CUDA;
  return AFV_OK;
}

// gsrb_boxes (src/m_aX_mg.f90:397-420): each half-sweep, then the level's
// ghost fill.
void Forest::gen_gsrb_boxes(int lvl, int n_cycle) {
  const int nbx = lvl_n(lvl);
  if (!nbx || n_cycle <= 0) return;
  const dev::Meta m = meta_for(meta);
  for (int n = 1; n <= 2 * n_cycle; ++n) {
    with_nc_op(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      opdev::k_gsrb<D, NC><<<grid_n((long long)nbx * G::SI / 2, n_sm), 256, 0, stream>>>(
          m, level_set(lvl), d64.phi, d64.rhs, eps_ptr(), d_tags, op, n);
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
  with_nc_op(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_restrict<D, NC><<<grid_n((long long)nbx * G::SI / (1 << D), n_sm), 256, 0, stream>>>(
        m, level_set(lvl), d64.phi, d64.rhs, d64.tmp, eps_ptr(), d_tags, op, lvl, copy_tmp ? 0 : 1);
    ++n_launches;
  });
  fill64(lvl - 1);
  const int np = n_parents(lvl - 1);
  if (!np) return;
  with_nc_op(plan.dim, plan.nc_at(lvl - 1), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_coarse<D, NC><<<grid_n((long long)np * G::SG, n_sm), 256, 0, stream>>>(
        m, dev::BoxSet{parents_list(lvl - 1), 0, np, 0, 0}, d64.phi, d64.rhs, d64.tmp, eps_ptr(), d_tags, op,
        copy_tmp ? 1 : 0);
    ++n_launches;
  });
}

// correct_children on the parents of level lp (src/m_aX_mg.f90:368-395).
void Forest::gen_correct(int lp) {
  const int np = n_parents(lp);
  if (!np) return;
  const dev::Meta m = meta_for(meta);
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
    opdev::k_correct<D, NC><<<grid_n((long long)np * nch * G::SI, n_sm), 256, 0, stream>>>(
        m, pb, nch, d64.phi, d64.tmp, eps_ptr(), d_tags, op, lp + 1);
    ++n_launches;
  });
}

// residual_box on every box of a level; with norm, max |tmp| over the leaves
// per tree into the striped norms.
void Forest::gen_residual(int lvl, unsigned long long* norm) {
  const int nbx = lvl_n(lvl);
  if (!nbx) return;
  const dev::Meta m = meta_for(meta);
  with_nc_op(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    opdev::k_residual<D, NC><<<grid_n((long long)nbx * G::SI, n_sm), 256, 0, stream>>>(
        m, level_set(lvl), d64.phi, d64.rhs, d64.tmp, eps_ptr(), d_tags, op);
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
