// The coarse end of the mixed solve's FP32 correction cycle in one block per
// tree (k_coarse_end).
//
// On the levels l0..1 every tree of a forest built with coarsen_to has one
// box per level (the base box and its coarsened copies, src/m_aX_core.f90:
// 74-83). There the V-cycle (src/m_aX_mg.f90:208-255) runs about fifteen
// launches per cycle -- half-sweeps, restriction, coarse right-hand side,
// the FP64 base smoothing with its conversions, correction -- each a few
// microseconds of launch and L2 latency for a few hundred cells. k_coarse_end
// runs all of them for one tree in one block, with the levels in static
// shared memory: from the down-leg sweeps of level 1 to the up-leg sweeps of
// level 1. Every operator computes the values its kernel computes, in the
// same order and precision:
//  * half-sweeps as k_sweep_small (ghosts pulled before each colour),
//  * restriction as k_restrict_res<SUB> (all face ghosts pulled, residual
//    and phi restricted into the parent's interior),
//  * coarse right-hand side as k_coarse_rhs (ghosts pulled and kept,
//    rhs = L phi + tmp, tmp = phi over the whole box),
//  * the base level in FP64 (converted in, n_base cycles, face ghosts
//    filled, converted back) as the base64 branch of the V-cycle,
//  * correction as k_correct<SUB> (ghosts pulled when the launch would pull
//    them, tmp = phi - tmp over the whole box, phi += prolong2(tmp)).
// Only level 1's interior is written back: the levels below it are scratch
// of the correction cycle (rewritten by restriction before their next use),
// and level 1's other values do not change between these operators.
// Homogeneous boundary conditions only (the correction cycle's).
#pragma once
#include "kernels.cuh"

namespace afv {
namespace dev {

constexpr int kCoarseEndThreads = 256;
constexpr int kCoarseEndMaxLevels = 4;  // level 1 and up to three coarsened copies

// One level of one tree in shared memory: a single box.
template <int D, int NC>
struct CeLevel {
  using G = Geo<D, NC>;
  float phi[G::SG];
  float tmp[G::SG];
  float rhs[G::SI];
};

// Cells of a level at depth L below level 1 (NC halves per level, at least 2).
template <int NC, int L>
struct CeNc {
  static constexpr int value = (NC >> L) >= 2 ? (NC >> L) : 2;
  static constexpr bool valid = (NC >> L) >= 2;
};

// Ghost value of face cell (f, a, c) of a single-box level under homogeneous
// boundary conditions: the box's own cell across a periodic face, else
// bc_to_gc with a zero boundary value.
template <int D, int NC, class T>
__device__ __forceinline__ T ce_ghost(const SlotDesc& d, const T* bx, int f, int a, int c, T dr) {
  using G = Geo<D, NC>;
  const Face<D, NC> F(f, a, c);
  const int code = d.code[f];
  if (code >= 0) return bx[G::g(F.ni, F.nj, F.nk)];
  return bc_value<T>(code, f, (T)0, bx[G::g(F.ai, F.aj, F.ak)], dr);
}

// All face ghosts of a level (pull_all_ghosts on a single box).
template <int D, int NC, class T>
__device__ void ce_fill(const SlotDesc& d, T* bx, T dr) {
  using G = Geo<D, NC>;
  for (int e = threadIdx.x; e < G::NNB * G::NF; e += blockDim.x) {
    const int f = e / G::NF, lin = e % G::NF;
    const int a = lin % NC + 1, c = lin / NC + 1;
    const Face<D, NC> F(f, a, c);
    const T v = ce_ghost<D, NC, T>(d, bx, f, a, c, dr);
    bx[G::g(F.gi, F.gj, F.gk)] = v;
  }
  __syncthreads();
}

// Half-sweeps n_first .. n_first + n_count - 1 (k_sweep_small's order).
template <int D, int NC, class T>
__device__ void ce_sweeps(const SlotDesc& d, T* bx, const T* rh, int n_first, int n_count, bool pull_first,
                          T dr, T dx2) {
  using G = Geo<D, NC>;
  constexpr int OX = 1, OY = G::NG, OZ = G::NG * G::NG;
  constexpr int HF = G::NF / 2;
  for (int h = 0; h < n_count; ++h) {
    const int nsw = n_first + h;
    if (h > 0 || pull_first) {
      for (int e = threadIdx.x; e < G::NNB * HF; e += blockDim.x) {
        const int f = e / HF, mcell = e % HF;
        int a, c;
        needed_face_cell<D, NC>(f, mcell, nsw, a, c);
        const Face<D, NC> F(f, a, c);
        const T v = ce_ghost<D, NC, T>(d, bx, f, a, c, dr);
        bx[G::g(F.gi, F.gj, F.gk)] = v;
      }
      __syncthreads();
    }
    for (int q = threadIdx.x; q < G::SI / 2; q += blockDim.x) {
      const int p = q % (NC / 2);
      int upos, rpos;
      if constexpr (D == 2) {
        const int j = q / (NC / 2) + 1;
        const int i = 2 * p + 1 + ((1 + j + nsw) & 1);
        upos = G::g(i, j, 0);
        rpos = G::in(i, j, 1);
      } else {
        const int j = (q / (NC / 2)) % NC + 1;
        const int k = q / ((NC / 2) * NC) + 1;
        const int i = 2 * p + 1 + ((1 + j + k + nsw) & 1);
        upos = G::g(i, j, k);
        rpos = G::in(i, j, k);
      }
      T* b = bx + upos;
      const T f = rh[rpos];
      T v;
      if constexpr (D == 2) {
        v = (T)0.25 * (b[OX] + b[-OX] + b[OY] + b[-OY] - dx2 * f);
      } else {
        const T sixth = (T)(1 / 6.0);
        v = sixth * (b[OX] + b[-OX] + b[OY] + b[-OY] + b[OZ] + b[-OZ] - dx2 * f);
      }
      *b = v;
    }
    __syncthreads();
  }
}

// Residual of the fine box restricted into its parent's tmp, phi into the
// parent's phi (k_restrict_res<SUB>: the parent covers the box with half the
// cells). The fine box's face ghosts are pulled first.
template <int D, int NC>
__device__ void ce_restrict(const SlotDesc& d, float* bx, const float* rh, float* pphi, float* ptmp) {
  using G = Geo<D, NC>;
  using GP = Geo<D, NC / 2>;
  constexpr int H = NC / 2;
  constexpr int PAR = D == 2 ? H * H : H * H * H;
  ce_fill<D, NC, float>(d, bx, d.drf);
  const float inv = d.inv_dx2f;
  for (int q = threadIdx.x; q < PAR; q += blockDim.x) {
    const int ic = q % H + 1, jc = (q / H) % H + 1, kc = (D == 3) ? q / (H * H) + 1 : 0;
    float sr = 0, sp = 0;
    constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
    for (int kk = 0; kk < KK; ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii) {
          const int i = 2 * ic - 1 + ii, j = 2 * jc - 1 + jj, k = (D == 3) ? 2 * kc - 1 + kk : 0;
          const float r = rh[G::in(i, j, k)] - lpl_at<D, NC, float>(bx, i, j, k, inv);
          sr = sr + r;
          sp = sp + bx[G::g(i, j, k)];
        }
    const float w = (D == 2) ? 0.25f : 0.125f;
    const int po = GP::g(ic, jc, (D == 3) ? kc : 0);
    ptmp[po] = w * sr;
    pphi[po] = w * sp;
  }
  __syncthreads();
}

// Coarse right-hand side of a parent (k_coarse_rhs with copy_tmp and pull):
// ghosts pulled and kept, rhs = L phi + tmp, then tmp = phi over the box.
template <int D, int NC>
__device__ void ce_coarse_rhs(const SlotDesc& d, float* bx, float* rh, float* tm) {
  using G = Geo<D, NC>;
  ce_fill<D, NC, float>(d, bx, d.drf);
  const float inv = d.inv_dx2f;
  for (int q = threadIdx.x; q < G::SI; q += blockDim.x) {
    const int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
    const float l = lpl_at<D, NC, float>(bx, i, j, k, inv);
    rh[q] = l + tm[G::g(i, j, k)];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < G::SG; e += blockDim.x) tm[e] = bx[e];
  __syncthreads();
}

// Correction of the child from its parent (k_correct<SUB>, the parent has
// NC cells per side, the child 2 NC): with pull the parent's face ghosts are
// recomputed and kept; tmp = phi - tmp over the parent's whole box; the
// child's interior gets prolong2(tmp) added.
template <int D, int NC>
__device__ void ce_correct(const SlotDesc& dp, float* pphi, float* ptmp, float* cphi, bool pull) {
  using G = Geo<D, NC>;
  using GC = Geo<D, 2 * NC>;
  if (pull) ce_fill<D, NC, float>(dp, pphi, dp.drf);
  for (int e = threadIdx.x; e < G::SG; e += blockDim.x) ptmp[e] = pphi[e] - ptmp[e];
  __syncthreads();
  const float* t = ptmp;
  for (int q = threadIdx.x; q < G::SI; q += blockDim.x) {
    const int ic = q % NC + 1, jc = (q / NC) % NC + 1, kc = (D == 3) ? q / (NC * NC) + 1 : 0;
    const int i_f = 2 * ic - 1, j_f = 2 * jc - 1;
    const float f0 = t[G::g(ic, jc, kc)];
    const float fx = 0.125f * (t[G::g(ic + 1, jc, kc)] - t[G::g(ic - 1, jc, kc)]);
    const float fy = 0.125f * (t[G::g(ic, jc + 1, kc)] - t[G::g(ic, jc - 1, kc)]);
    const float fxx = 0.03125f * (t[G::g(ic - 1, jc, kc)] - 2.0f * f0 + t[G::g(ic + 1, jc, kc)]);
    const float fyy = 0.03125f * (t[G::g(ic, jc - 1, kc)] - 2.0f * f0 + t[G::g(ic, jc + 1, kc)]);
    if constexpr (D == 2) {
      const float f2 = fxx + fyy;
      const int o00 = GC::g(i_f, j_f, 0), o10 = GC::g(i_f + 1, j_f, 0);
      const int o01 = GC::g(i_f, j_f + 1, 0), o11 = GC::g(i_f + 1, j_f + 1, 0);
      cphi[o00] = f0 - fx - fy + f2 + cphi[o00];
      cphi[o10] = f0 + fx - fy + f2 + cphi[o10];
      cphi[o01] = f0 - fx + fy + f2 + cphi[o01];
      cphi[o11] = f0 + fx + fy + f2 + cphi[o11];
    } else {
      const int k_f = 2 * kc - 1;
      const float fz = 0.125f * (t[G::g(ic, jc, kc + 1)] - t[G::g(ic, jc, kc - 1)]);
      const float fzz = 0.03125f * (t[G::g(ic, jc, kc - 1)] - 2.0f * f0 + t[G::g(ic, jc, kc + 1)]);
      const float f2 = fxx + fyy + fzz;
#pragma unroll
      for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
          for (int cx = 0; cx < 2; ++cx) {
            const int o = GC::g(i_f + cx, j_f + cy, k_f + cz);
            float v = f0;
            v = cx ? v + fx : v - fx;
            v = cy ? v + fy : v - fy;
            v = cz ? v + fz : v - fz;
            cphi[o] = v + f2 + cphi[o];
          }
    }
  }
  __syncthreads();
}

// The base level in FP64 (the base64 branch of the V-cycle): phi and rhs
// converted to FP64, n_base cycles of half-sweeps (ghosts pulled), all face
// ghosts filled, phi converted back over the whole box.
template <int D, int NC>
__device__ void ce_base64(const SlotDesc& d, float* bx, const float* rh, double* b64, double* r64, int n_base) {
  using G = Geo<D, NC>;
  for (int e = threadIdx.x; e < G::SG; e += blockDim.x) b64[e] = (double)bx[e];
  for (int e = threadIdx.x; e < G::SI; e += blockDim.x) r64[e] = (double)rh[e];
  __syncthreads();
  if (n_base > 0) {
    ce_sweeps<D, NC, double>(d, b64, r64, 1, 2 * n_base, true, d.dr, d.dx2);
    ce_fill<D, NC, double>(d, b64, d.dr);
  }
  for (int e = threadIdx.x; e < G::SG; e += blockDim.x) bx[e] = (float)b64[e];
  __syncthreads();
}

// First slot of each level 1, 0, -1, ... (the tree's box is first + tree).
struct CeSlots {
  int lo[kCoarseEndMaxLevels];
};

// The NL levels 1 .. 2 - NL of one tree, the FP64 copy of the base level and
// the levels' descriptors, in static shared memory (about 14 KB for 8^3
// boxes with two coarsened levels).
template <int D, int NC, int NL>
struct CeStore {
  CeLevel<D, CeNc<NC, 0>::value> v0;
  CeLevel<D, CeNc<NC, 1>::value> v1;
  CeLevel<D, CeNc<NC, 2>::value> v2;
  CeLevel<D, CeNc<NC, 3>::value> v3;
  double b64[Geo<D, CeNc<NC, NL - 1>::value>::SG];
  double r64[Geo<D, CeNc<NC, NL - 1>::value>::SI];
  SlotDesc sd[kCoarseEndMaxLevels];
};

template <int L, class S>
__device__ __forceinline__ auto& ce_lv(S& s) {
  if constexpr (L == 0)
    return s.v0;
  else if constexpr (L == 1)
    return s.v1;
  else if constexpr (L == 2)
    return s.v2;
  else
    return s.v3;
}

// Down leg from depth L (level 1 - L): sweeps, restriction, coarse rhs.
template <int D, int NC, int NL, int L>
__device__ void ce_down(CeStore<D, NC, NL>& s, int n_down) {
  if constexpr (L < NL - 1) {
    constexpr int N = CeNc<NC, L>::value;
    auto& a = ce_lv<L>(s);
    auto& p = ce_lv<L + 1>(s);
    const SlotDesc& d = s.sd[L];
    if (n_down > 0) ce_sweeps<D, N, float>(d, a.phi, a.rhs, 1, 2 * n_down, true, d.drf, d.dx2f);
    ce_restrict<D, N>(d, a.phi, a.rhs, p.phi, p.tmp);
    ce_coarse_rhs<D, N / 2>(s.sd[L + 1], p.phi, p.rhs, p.tmp);
    ce_down<D, NC, NL, L + 1>(s, n_down);
  }
}

// Up leg at depth L (level 1 - L): correction from the level below, sweeps.
template <int D, int NC, int NL, int L>
__device__ void ce_up(CeStore<D, NC, NL>& s, int n_up) {
  if constexpr (L >= 0 && L < NL - 1) {
    constexpr int N = CeNc<NC, L>::value;
    auto& a = ce_lv<L>(s);
    auto& p = ce_lv<L + 1>(s);
    const SlotDesc& d = s.sd[L];
    // the launch pulls the parent's ghosts unless the parent is the base level
    ce_correct<D, N / 2>(s.sd[L + 1], p.phi, p.tmp, a.phi, L + 1 < NL - 1);
    if (n_up > 0) ce_sweeps<D, N, float>(d, a.phi, a.rhs, 1, 2 * n_up, true, d.drf, d.dx2f);
    ce_up<D, NC, NL, L - 1>(s, n_up);
  }
}

template <int D, int NC, int NL>
__global__ void __launch_bounds__(kCoarseEndThreads)
k_coarse_end(Meta m, CeSlots sl, float* __restrict__ phi, const float* __restrict__ rhs, int n_down, int n_up,
             int n_base) {
  static_assert(NL >= 1 && NL <= kCoarseEndMaxLevels && (NC >> (NL - 1)) >= 2, "coarse-end levels");
  pdl_trigger();
  __shared__ __align__(16) CeStore<D, NC, NL> s;
  const int t = blockIdx.x;
  // descriptors never change: copied before the wait
  for (int e = threadIdx.x; e < NL * (int)(sizeof(SlotDesc) / 4); e += blockDim.x) {
    const int l = e / (int)(sizeof(SlotDesc) / 4), w = e % (int)(sizeof(SlotDesc) / 4);
    reinterpret_cast<unsigned*>(&s.sd[l])[w] = reinterpret_cast<const unsigned*>(m.desc + sl.lo[l] + t)[w];
  }
  pdl_wait();
  if (!m.active[t]) return;  // the whole block: one tree
  __syncthreads();
  using G0 = Geo<D, NC>;
  auto& top = s.v0;
  {
    const float* src = phi + s.sd[0].offg;
    for (int e = threadIdx.x; e < G0::SG; e += blockDim.x) top.phi[e] = src[e];
    const float* r = rhs + s.sd[0].offi;
    for (int e = threadIdx.x; e < G0::SI; e += blockDim.x) top.rhs[e] = r[e];
  }
  // the coarsened levels start from zero (every value read is written first)
  auto zero = [&](auto& v) {
    constexpr int SG = (int)(sizeof(v.phi) / sizeof(float));
    for (int e = threadIdx.x; e < SG; e += blockDim.x) v.phi[e] = v.tmp[e] = 0.f;
  };
  if constexpr (NL > 1) zero(s.v1);
  if constexpr (NL > 2) zero(s.v2);
  if constexpr (NL > 3) zero(s.v3);
  __syncthreads();
  ce_down<D, NC, NL, 0>(s, n_down);
  {
    constexpr int NB = CeNc<NC, NL - 1>::value;
    auto& b = ce_lv<NL - 1>(s);
    ce_base64<D, NB>(s.sd[NL - 1], b.phi, b.rhs, s.b64, s.r64, n_base);
  }
  ce_up<D, NC, NL, NL - 2>(s, n_up);
  float* dst = phi + s.sd[0].offg;
  for (int q = threadIdx.x; q < G0::SI; q += blockDim.x) {
    const int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
    dst[G0::g(i, j, k)] = top.phi[G0::g(i, j, k)];
  }
}

}  // namespace dev
}  // namespace afv
