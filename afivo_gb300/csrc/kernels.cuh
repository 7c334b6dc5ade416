// Device kernels of the FAS multigrid path (sm_103a). Templated on the
// dimension D, the block size NC of the level they sweep and the arithmetic
// type T (double for the FP64 path, float for the inner cycles of the mixed
// path).
//
// Storage: every variable is one flat device array shared by all levels and
// trees; slot s keeps phi/tmp at offg[s] as a (NC+2)^D box with one ghost
// layer, x fastest (the reference's cc(0:nc+1, ...) arrays,
// src/m_aX_core.f90:360-369), and rhs at offi[s] as an NC^D interior-only box
// (rhs ghost cells are never read by the reference's path). A 128-byte
// SlotDesc per slot (desc.hpp) holds the box's links and constants.
//
// Floating-point order follows the reference expression by expression; the
// library is compiled with -fmad=false so that no multiply-add is fused
// (the mixed path's FP64 defect uses explicit fma() where stated).
#pragma once
#include <cstdint>
#include <type_traits>

#include "desc.hpp"

namespace afv {
namespace dev {

constexpr int kThreads = 256;
constexpr int kSmemCap = 48 * 1024;

struct BoxSet {
  const int* list;  // slot list, or nullptr for the range [lo, lo+n)
  int lo;
  int n;
  long long g0, i0;  // range: offg and offi of slot lo (a level's boxes are stored
                     // consecutively, so box i of the range is at g0 + i * SG)
};

struct Meta {
  const int* tree;         // [slot]
  const int* parent;       // [slot]
  const int* first_child;  // [slot]
  const long long* offg;   // [slot] offset of the ghosted box
  const long long* offi;   // [slot] offset of the interior box
  const double* bcval;     // boundary values (faces of physical boundaries)
  const int* active;       // [tree] nonzero if the tree takes part in this launch
  const SlotDesc* desc;    // [slot]
  const long long* nbo2;   // [slot*2D + face] refinement boundary: offg of the parent's neighbour
  int* err;                // device error word: nonzero after a bounded wait gave up
  long long wait_limit;    // clock cycles a wait for a copy may take before it gives up;
                           // <= 0: give up at once (exercises the error path)
};

__device__ __forceinline__ int box_at(const BoxSet& s, int i) { return s.list ? s.list[i] : s.lo + i; }
// Storage offsets of box i (slot s) of a set: arithmetic for ranges, a table
// load for lists.
template <int SG>
__device__ __forceinline__ long long box_offg(const Meta& m, const BoxSet& bs, int i, int s) {
  return bs.list ? m.offg[s] : bs.g0 + (long long)i * SG;
}
template <int SI>
__device__ __forceinline__ long long box_offi(const Meta& m, const BoxSet& bs, int i, int s) {
  return bs.list ? m.offi[s] : bs.i0 + (long long)i * SI;
}

template <int D, int NC>
struct Geo {
  static constexpr int NG = NC + 2;
  static constexpr int SG = D == 2 ? NG * NG : NG * NG * NG;
  static constexpr int SI = D == 2 ? NC * NC : NC * NC * NC;
  static constexpr int NF = D == 2 ? NC : NC * NC;
  static constexpr int NNB = 2 * D;
  __host__ __device__ static constexpr int g(int i, int j, int k) { return i + NG * (j + NG * k); }
  // interior index; k is ignored in 2-D
  __host__ __device__ static constexpr int in(int i, int j, int k) {
    return (i - 1) + NC * ((j - 1) + (D == 3 ? NC * (k - 1) : 0));
  }
};

template <class T> struct Vec;
template <> struct Vec<double> { using type = double2; static constexpr int w = 2; };
template <> struct Vec<float> { using type = float4; static constexpr int w = 4; };

// Per-precision constants of a slot.
template <class T> struct Sc;
template <> struct Sc<double> {
  __device__ static double dr(const SlotDesc& d) { return d.dr; }
  __device__ static double dx2(const SlotDesc& d) { return d.dx2; }
  __device__ static double inv(const SlotDesc& d) { return d.inv_dx2; }
};
template <> struct Sc<float> {
  __device__ static float dr(const SlotDesc& d) { return d.drf; }
  __device__ static float dx2(const SlotDesc& d) { return d.dx2f; }
  __device__ static float inv(const SlotDesc& d) { return d.inv_dx2f; }
};

template <int SG, int PER_BOX, class T>
__host__ __device__ constexpr int boxes_per_cta(int staged) {
  int by_threads = kThreads / PER_BOX;
  int by_smem = kSmemCap / (SG * (int)sizeof(T) * staged);
  int b = by_threads < by_smem ? by_threads : by_smem;
  return b < 1 ? 1 : b;
}

// Face cell (a, c) of face f (0-based: lowx, highx, lowy, highy, lowz, highz):
// ghost position, the adjacent interior cell, and the matching boundary cell
// of the neighbour across the face. a, c run over 1..NC in the tangential
// directions (x before y before z).
template <int D, int NC>
struct Face {
  int gi, gj, gk;  // ghost cell
  int ai, aj, ak;  // adjacent interior cell
  int ni, nj, nk;  // neighbour's cell copied into the ghost (sides_from_nb)
  __device__ __forceinline__ Face(int f, int a, int c) {
    const int hi = f & 1;
    const int gn = hi ? NC + 1 : 0, an = hi ? NC : 1, nn = hi ? 1 : NC;
    const int cz = (D == 3) ? c : 0;
    switch (f >> 1) {
      case 0:
        gi = gn; ai = an; ni = nn;
        gj = aj = nj = a;
        gk = ak = nk = cz;
        break;
      case 1:
        gj = gn; aj = an; nj = nn;
        gi = ai = ni = a;
        gk = ak = nk = cz;
        break;
      default:
        gk = gn; ak = an; nk = nn;
        gi = ai = ni = a;
        gj = aj = nj = c;
        break;
    }
  }
};

// Cell of the parent (or, two hops away, of the parent's neighbour) that the
// zeroth-order injection a$D_prolong0 (src/m_aX_prolong.f90:88-94) copies into
// ghost cell F of a box with child bits qd. With two_hop the parent's ghost
// cell is replaced by the neighbour's boundary cell it holds.
template <int D, int NC>
__device__ __forceinline__ int parent_cell(const Face<D, NC>& F, int f, int qd, bool two_hop) {
  const int h = NC >> 1;
  int pi = (qd & 1) * h + ((F.gi + 1) >> 1);
  int pj = ((qd >> 1) & 1) * h + ((F.gj + 1) >> 1);
  int pk = (D == 3) ? ((qd >> 2) & 1) * h + ((F.gk + 1) >> 1) : 0;
  if (two_hop) {  // ghost index 0 <- neighbour's NC, ghost index NC+1 <- neighbour's 1
    const int mirror = (f & 1) ? 1 : NC;
    switch (f >> 1) {
      case 0: pi = mirror; break;
      case 1: pj = mirror; break;
      default: pk = mirror; break;
    }
  }
  return Geo<D, NC>::g(pi, pj, pk);
}

// Ghost value from the injected parent value g0 and the box's own cells:
// mg$D_sides_rb, src/m_aX_mg.f90:286-347 (2-D and 3-D forms).
template <int D, int NC, class T, class Own>
__device__ __forceinline__ T rb_value(const Face<D, NC>& F, int f, T g0, Own own) {
  const int dim = f >> 1, dix = (f & 1) ? -1 : 1;
  const int i = F.ai, j = F.aj, k = F.ak;
  if constexpr (D == 2) {
    if (dim == 0) {
      const int dj = -1 + 2 * (j & 1);
      return (T)0.5 * g0 + own(i, j, 0) - (T)0.25 * (own(i + dix, j, 0) + own(i, j + dj, 0));
    } else {
      const int di = -1 + 2 * (i & 1);
      return (T)0.5 * g0 + own(i, j, 0) - (T)0.25 * (own(i + di, j, 0) + own(i, j + dix, 0));
    }
  } else {
    const int di = (dim == 0) ? dix : -1 + 2 * (i & 1);
    const int dj = (dim == 1) ? dix : -1 + 2 * (j & 1);
    const int dk = (dim == 2) ? dix : -1 + 2 * (k & 1);
    return (T)0.5 * g0 + (T)0.75 * own(i, j, k) - (T)0.25 * own(i + di, j + dj, k + dk);
  }
}

// Physical boundary, bc_to_gc (src/m_aX_gc.f90:71-132): y = c2 * b + c1 * x
// with (c1, c2) = (-1, 2) for Dirichlet and (1, dr * (+-1)) for Neumann.
template <class T>
__device__ __forceinline__ T bc_value(int code, int f, T b, T x, T dr) {
  if (code == kFaceDirichlet) return (T)2 * b + (T)(-1) * x;
  const T c2 = dr * (T)((f & 1) ? 1 : -1);
  return c2 * b + (T)1 * x;
}

// Ghost value of one face cell of a slot from the current state of its level
// (own(i,j,k) reads the box's own cells): the value the reference's a$D_gc_box
// (src/m_aX_gc.f90:50-69) stores there.
//  - neighbour box: copy of its boundary cell (sides_from_nb, :381-415)
//  - refinement boundary: parent injection + mg$D_sides_rb
//  - physical boundary: bc_to_gc with the sampled sides_bc value
template <int D, int NC, class T, class Own>
__device__ __forceinline__ T ghost_value(const Meta& m, const SlotDesc& d, const T* __restrict__ phi,
                                         int f, int a, int c, bool homog, Own own) {
  using G = Geo<D, NC>;
  const Face<D, NC> F(f, a, c);
  const int code = d.code[f];
  const long long o = d.nbo[f];
  if (code >= 0) return phi[o + G::g(F.ni, F.nj, F.nk)];
  if (code == kFaceRefinement) {
    const T g0 = phi[o + parent_cell<D, NC>(F, f, d.qd, false)];
    return rb_value<D, NC, T>(F, f, g0, own);
  }
  T b = 0;
  if (!homog && o >= 0) b = (T)m.bcval[o + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
  return bc_value<T>(code, f, b, own(F.ai, F.aj, F.ak), Sc<T>::dr(d));
}

// Programmatic dependent launch: every kernel may be scheduled while the
// previous kernel on its stream drains; pdl_wait() returns once that kernel
// has finished and its writes are visible, pdl_trigger() lets the next kernel
// be scheduled. Both are no-ops for a launch without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Bulk copies (TMA, cp.async.bulk) into shared memory, completed on mbarriers.
// Every wait is bounded by a clock budget (Meta::wait_limit, set per forest);
// a kernel that gives up records it in the error word and drains its own
// copies before it returns. The drain waits with the fixed kDrainLimitCycles,
// so that a short (or zero) wait limit still lets every copy in flight land
// before the block's shared memory is released.
// ---------------------------------------------------------------------------
constexpr long long kWaitLimitCycles = 4000000000LL;   // default limit, about two seconds
constexpr long long kDrainLimitCycles = 4000000000LL;  // drain after giving up

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Per-thread asynchronous 16-byte copies global -> shared (cp.async), grouped
// per thread and waited for with cp.async.wait_group.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// try_wait with a suspend-time hint (ns): the warp sleeps until the phase
// completes or the hint elapses instead of spinning.
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(20000u)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  long long limit) {
  if (limit <= 0) return false;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}

// The cell (a, c) on face f whose adjacent interior cell is updated by
// half-sweep n (the ghosts that sweep reads); m enumerates them.
template <int D, int NC>
__device__ __forceinline__ void needed_face_cell(int f, int m, int n, int& a, int& c) {
  const int an = (f & 1) ? NC : 1;
  if constexpr (D == 2) {
    c = 1;
    a = 2 * m + 1 + ((1 + an + n) & 1);
  } else {
    c = m / (NC / 2) + 1;
    a = 2 * (m % (NC / 2)) + 1 + ((1 + an + c + n) & 1);
  }
}

enum { kModeSweep = 0, kModeFill = 1 };

template <int D, int NC, class T, int MODE>
struct LevelCfg {
  using G = Geo<D, NC>;
  static constexpr int S = 6;                   // pipeline stages
  static constexpr int LA = S - 2;              // groups issued ahead of the one in use
  static constexpr bool SWEEP = MODE == kModeSweep;
  static constexpr int PER_BOX = G::SI / 2;     // sweep: one thread per updated cell
  static constexpr int NEED = SWEEP ? 2 * D * (G::NF / 2) : 2 * D * G::NF;  // ghost items per box
  static constexpr int BOX_B = (int)sizeof(SlotDesc) + (G::SG + (SWEEP ? G::SI : 0)) * (int)sizeof(T);
  static constexpr int BPC_T = SWEEP ? kThreads / PER_BOX : (2 * kThreads / NEED > 0 ? 2 * kThreads / NEED : 1);
  static constexpr int BPC_S = 100 * 1024 / (S * BOX_B);
  static constexpr int BPC = BPC_T < BPC_S ? BPC_T : (BPC_S < 1 ? 1 : BPC_S);
  static constexpr int ITEMS = (BPC * NEED + kThreads - 1) / kThreads;
  static constexpr int DESC_B = BPC * (int)sizeof(SlotDesc);
  static constexpr int PHI_B = BPC * G::SG * (int)sizeof(T);
  static constexpr int RHS_B = SWEEP ? BPC * G::SI * (int)sizeof(T) : 0;
  static constexpr int STAGE_B = DESC_B + PHI_B + RHS_B;
  static constexpr int SMEM_B = S * STAGE_B;  // dynamic shared memory
  static_assert(G::SG * sizeof(T) % 16 == 0 && G::SI * sizeof(T) % 16 == 0, "bulk copy sizes");
};

// ---------------------------------------------------------------------------
// Level kernel, persistent and pipelined, in two modes.
//
// kModeSweep -- GSRB half-sweep on every box of one level (mg$D_box_gsrb_lpl,
// src/m_aX_mg.f90:718-760). With pull = 1 the ghost cells this colour reads
// are the values of the a$D_gc_box fill the reference runs after the previous
// half-sweep (src/m_aX_mg.f90:412-417): neighbours' cells of the other colour,
// which no block writes during this sweep, so all blocks update in place. With
// pull = 0 the stored ghost cells are used (first half-sweep).
//
// kModeFill -- ghost fill of every face of every box of a set (a$D_gc_box,
// src/m_aX_gc.f90:50-69, as called by fill_gc_phi, src/m_aX_mg.f90:352-365):
// writes only ghost cells, reads only interior cells of the level and the
// parents' stored cells, so all boxes fill concurrently.
//
// Each block streams its groups of boxes through an S-stage ring in shared
// memory (bulk copies of descriptors, phi and rhs, issued LA groups ahead) and
// loads the ghost sources of the next group into registers while the current
// group is processed. One block barrier per group: the stage refilled at
// group k was last read at group k-2, which every thread finished before the
// barrier of group k-1. The colour is fixed per launch, so each thread's ghost
// items and updated cell -- and their index arithmetic -- are computed once.
// ---------------------------------------------------------------------------
template <int D, int NC, class T, int MODE>
__global__ void __launch_bounds__(kThreads)
k_level_tma(Meta m, BoxSet bs, T* __restrict__ phi, const T* __restrict__ rhs, int n, int pull, int homog) {
  pdl_wait();
  pdl_trigger();
  using C = LevelCfg<D, NC, T, MODE>;
  using G = Geo<D, NC>;
  constexpr int S = C::S;
  constexpr bool SWEEP = C::SWEEP;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar[S];
  __shared__ int s_act[S][C::BPC];
  __shared__ int s_abort;
  if (!SWEEP) pull = 1;

  const int nbx = bs.n;
  const int groups = (nbx + C::BPC - 1) / C::BPC;
  if ((int)blockIdx.x >= groups) return;
  const int my_groups = (groups - 1 - (int)blockIdx.x) / (int)gridDim.x + 1;

  if (threadIdx.x == 0) {
    for (int st = 0; st < S; ++st) mbar_init(&bar[st], 1);
    s_abort = 0;
    fence_mbar_init();
  }

  // Per-thread constants of the ghost items.
  int it_b[C::ITEMS], it_f[C::ITEMS], it_gpos[C::ITEMS], it_npos[C::ITEMS], it_apos[C::ITEMS];
  int it_lin[C::ITEMS];
  short it_gi[C::ITEMS], it_gj[C::ITEMS], it_gk[C::ITEMS];
#pragma unroll
  for (int j = 0; j < C::ITEMS; ++j) {
    const int e = threadIdx.x + j * kThreads;
    it_b[j] = e / C::NEED;  // box within the group (>= BPC: no item)
    const int r = e % C::NEED;
    int f, a, c;
    if constexpr (SWEEP) {
      f = r / (G::NF / 2);
      needed_face_cell<D, NC>(f, r % (G::NF / 2), n, a, c);
    } else {
      f = r / G::NF;
      const int lin = r % G::NF;
      a = lin % NC + 1;
      c = lin / NC + 1;
    }
    const Face<D, NC> F(f, a, c);
    it_f[j] = f;
    it_gpos[j] = G::g(F.gi, F.gj, F.gk);
    it_npos[j] = G::g(F.ni, F.nj, F.nk);
    it_apos[j] = G::g(F.ai, F.aj, F.ak);
    it_lin[j] = (D == 2) ? (a - 1) : (a - 1) + NC * (c - 1);
    it_gi[j] = (short)F.gi;
    it_gj[j] = (short)F.gj;
    it_gk[j] = (short)F.gk;
  }
  // Sweep: the cell this thread updates.
  const int ub = threadIdx.x / C::PER_BOX, uq = threadIdx.x % C::PER_BOX;
  int upos = 0, rpos = 0;
  if constexpr (SWEEP) {
    const int p = uq % (NC / 2);
    if constexpr (D == 2) {
      const int j = uq / (NC / 2) + 1;
      const int i = 2 * p + 1 + ((1 + j + n) & 1);
      upos = G::g(i, j, 0);
      rpos = G::in(i, j, 1);
    } else {
      const int j = (uq / (NC / 2)) % NC + 1;
      const int k = uq / ((NC / 2) * NC) + 1;
      const int i = 2 * p + 1 + ((1 + j + k + n) & 1);
      upos = G::g(i, j, k);
      rpos = G::in(i, j, k);
    }
  }
  constexpr int OX = 1, OY = G::NG, OZ = G::NG * G::NG;
  __syncthreads();

  auto group_first = [&](int k) { return ((int)blockIdx.x + k * (int)gridDim.x) * C::BPC; };
  auto group_n = [&](int k) { return min(C::BPC, nbx - group_first(k)); };
  auto issue = [&](int k) {  // one thread
    const int first = group_first(k), nb = group_n(k);
    unsigned char* sp = smem + (k % S) * C::STAGE_B;
    unsigned long long* b = &bar[k % S];
    fence_proxy_async();
    mbar_expect_tx(b, nb * (unsigned)C::BOX_B);
    if (!bs.list) {  // consecutive slots: consecutive storage
      const int s0 = bs.lo + first;
      bulk_g2s(sp, m.desc + s0, nb * (unsigned)sizeof(SlotDesc), b);
      bulk_g2s(sp + C::DESC_B, phi + bs.g0 + (long long)first * G::SG, nb * (unsigned)(G::SG * sizeof(T)), b);
      if constexpr (SWEEP)
        bulk_g2s(sp + C::DESC_B + C::PHI_B, rhs + bs.i0 + (long long)first * G::SI,
                 nb * (unsigned)(G::SI * sizeof(T)), b);
    } else {
      for (int q = 0; q < nb; ++q) {
        const int s = bs.list[first + q];
        bulk_g2s(sp + q * sizeof(SlotDesc), m.desc + s, (unsigned)sizeof(SlotDesc), b);
        bulk_g2s(sp + C::DESC_B + q * G::SG * sizeof(T), phi + m.offg[s], (unsigned)(G::SG * sizeof(T)), b);
        if constexpr (SWEEP)
          bulk_g2s(sp + C::DESC_B + C::PHI_B + q * G::SI * sizeof(T), rhs + m.offi[s],
                   (unsigned)(G::SI * sizeof(T)), b);
      }
    }
  };
  // Ghost sources of group k (its stage has landed): neighbour cells, parent
  // cells at refinement boundaries, or boundary values.
  auto prefetch = [&](int k, T (&val)[C::ITEMS], int& act) {
    const SlotDesc* dsc = reinterpret_cast<const SlotDesc*>(smem + (k % S) * C::STAGE_B);
    const int nb = group_n(k);
    act = ((int)threadIdx.x < nb) ? m.active[dsc[threadIdx.x].tree] : 0;
#pragma unroll
    for (int j = 0; j < C::ITEMS; ++j) {
      val[j] = (T)0;
      if (!pull || it_b[j] >= nb) continue;
      const SlotDesc& d = dsc[it_b[j]];
      const int f = it_f[j];
      const int code = d.code[f];
      const long long o = d.nbo[f];
      if (code >= 0) {
        val[j] = phi[o + it_npos[j]];
      } else if (code == kFaceRefinement) {
        const int h = NC >> 1, qd = d.qd;
        const int pi = (qd & 1) * h + ((it_gi[j] + 1) >> 1);
        const int pj = ((qd >> 1) & 1) * h + ((it_gj[j] + 1) >> 1);
        const int pk = (D == 3) ? ((qd >> 2) & 1) * h + ((it_gk[j] + 1) >> 1) : 0;
        val[j] = phi[o + G::g(pi, pj, pk)];
      } else if (o >= 0 && !homog) {
        val[j] = (T)m.bcval[o + it_lin[j]];
      }
    }
  };

  int issued = min(C::LA, my_groups);
  if (threadIdx.x == 0)
    for (int k = 0; k < issued; ++k) issue(k);

  // Returns false when the block has to stop (a bounded wait gave up).
  auto body = [&](int k, T (&cur)[C::ITEMS], int& cur_act, T (&nxt)[C::ITEMS], int& nxt_act) -> bool {
    const int st = k % S;
    unsigned char* sp = smem + st * C::STAGE_B;
    const SlotDesc* dsc = reinterpret_cast<const SlotDesc*>(sp);
    T* sphi = reinterpret_cast<T*>(sp + C::DESC_B);
    const int nb = group_n(k);
    if (k + C::LA < my_groups) {
      if (threadIdx.x == 0) issue(k + C::LA);
      ++issued;
    }
    if (k + 1 < my_groups) {
      if (mbar_wait_bounded(&bar[(k + 1) % S], ((k + 1) / S) & 1, m.wait_limit))
        prefetch(k + 1, nxt, nxt_act);
      else
        s_abort = 1;
    }
    if ((int)threadIdx.x < nb) s_act[st][threadIdx.x] = cur_act;
    if (pull) {
#pragma unroll
      for (int j = 0; j < C::ITEMS; ++j) {
        if (it_b[j] >= nb) continue;
        const SlotDesc& d = dsc[it_b[j]];
        if (!SWEEP && !m.active[d.tree]) continue;
        const int f = it_f[j];
        const int code = d.code[f];
        T* bx = sphi + it_b[j] * G::SG;
        T v = cur[j];
        if (code < 0) {  // boundary: formula from the box's own cells
          if (code == kFaceRefinement) {  // mg$D_sides_rb, src/m_aX_mg.f90:286-347
            const int dix = (f & 1) ? -1 : 1;
            const int ap = it_apos[j];
            const int dim = f >> 1;
            if constexpr (D == 2) {
              // x-direction term first, then the y-direction term; the
              // tangential step alternates with the tangential index
              if (dim == 0) {
                const int dj = -1 + 2 * ((int)it_gj[j] & 1);
                v = (T)0.5 * cur[j] + bx[ap] - (T)0.25 * (bx[ap + dix * OX] + bx[ap + dj * OY]);
              } else {
                const int di = -1 + 2 * ((int)it_gi[j] & 1);
                v = (T)0.5 * cur[j] + bx[ap] - (T)0.25 * (bx[ap + di * OX] + bx[ap + dix * OY]);
              }
            } else {
              const int ti = (int)it_gi[j], tj = (int)it_gj[j], tk = (int)it_gk[j];
              const int di = (dim == 0) ? dix : -1 + 2 * (ti & 1);
              const int dj = (dim == 1) ? dix : -1 + 2 * (tj & 1);
              const int dk = (dim == 2) ? dix : -1 + 2 * (tk & 1);
              v = (T)0.5 * cur[j] + (T)0.75 * bx[ap] - (T)0.25 * bx[ap + di * OX + dj * OY + dk * OZ];
            }
          } else {
            v = bc_value<T>(code, f, cur[j], bx[it_apos[j]], Sc<T>::dr(d));
          }
        }
        if constexpr (SWEEP)
          bx[it_gpos[j]] = v;
        else
          phi[d.offg + it_gpos[j]] = v;
      }
    }
    __syncthreads();
    if (s_abort) return false;
    if constexpr (SWEEP) {
      const T* srhs = reinterpret_cast<const T*>(sp + C::DESC_B + C::PHI_B);
      if (ub < nb && s_act[st][ub]) {
        const T* bx = sphi + ub * G::SG + upos;
        const SlotDesc& d = dsc[ub];
        const T f = srhs[ub * G::SI + rpos];
        T v;
        if constexpr (D == 2) {
          v = (T)0.25 * (bx[OX] + bx[-OX] + bx[OY] + bx[-OY] - Sc<T>::dx2(d) * f);
        } else {
          const T sixth = (T)(1 / 6.0);
          v = sixth * (bx[OX] + bx[-OX] + bx[OY] + bx[-OY] + bx[OZ] + bx[-OZ] - Sc<T>::dx2(d) * f);
        }
        phi[d.offg + upos] = v;
      }
    }
    return true;
  };

  T ra[C::ITEMS], rb[C::ITEMS];
  int act_a = 0, act_b = 0;
  bool ok = mbar_wait_bounded(&bar[0], 0, m.wait_limit);
  if (ok) prefetch(0, ra, act_a);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) {
      atomicExch(m.err, 1);
      for (int k = 0; k < issued; ++k) mbar_wait_bounded(&bar[k % S], (k / S) & 1, kDrainLimitCycles);
    }
    return;
  }
  int k = 0;
  for (; k < my_groups; k += 2) {
    if (!body(k, ra, act_a, rb, act_b)) break;
    if (k + 1 < my_groups && !body(k + 1, rb, act_b, ra, act_a)) {
      k += 1;
      break;
    }
  }
  if (k < my_groups && threadIdx.x == 0) {  // gave up: drain this block's copies
    atomicExch(m.err, 1);
    for (int j = k + 1; j < issued; ++j) mbar_wait_bounded(&bar[j % S], (j / S) & 1, kDrainLimitCycles);
  }
}

// ---------------------------------------------------------------------------
// Warp-per-box GSRB half-sweep (mg$D_box_gsrb_lpl, src/m_aX_mg.f90:718-760).
//
// Each warp owns a ring of S shared-memory stages and streams its own boxes
// (global warp w takes boxes w, w + total warps, ...) through it: lane 0
// issues the bulk copies of descriptor and phi S-1 boxes ahead, and all lanes
// wait on the stage's mbarrier. No block barrier: the warp's lanes pull the
// ghost cells this colour reads into the staged box (the same values as in
// k_level_tma), __syncwarp, then update the box's cells of the colour (CPL per
// lane) and store them. The ghost sources and the rhs values of a box are
// loaded into registers two boxes ahead, from its descriptor read straight
// from global memory four boxes ahead, so no load latency sits on the path.
// ---------------------------------------------------------------------------
template <int D, int NC, class T, int W, int S>
struct WarpCfg {
  using G = Geo<D, NC>;
  static constexpr int UPD = G::SI / 2;             // cells of one colour
  static constexpr int CPL = (UPD + 31) / 32;       // per lane
  static constexpr int NEED = 2 * D * (G::NF / 2);  // ghost cells this colour reads
  static constexpr int GPL = (NEED + 31) / 32;      // per lane
  static constexpr int PHI_OFF = (int)sizeof(SlotDesc);
  static constexpr int BOX_B = PHI_OFF + G::SG * (int)sizeof(T);  // rhs goes to registers
  static constexpr int SMEM_B = W * S * BOX_B;
  static_assert(BOX_B % 16 == 0, "bulk copy alignment");
};

// Fields of a SlotDesc held as one 32-bit word per lane (lane q: bytes 4q..4q+3).
struct DescWords {
  static __device__ __forceinline__ long long nbo(unsigned w, int f) {
    const unsigned lo = __shfl_sync(0xffffffffu, w, 2 * f);
    const unsigned hi = __shfl_sync(0xffffffffu, w, 2 * f + 1);
    return (long long)(((unsigned long long)hi << 32) | lo);
  }
  static __device__ __forceinline__ int code(unsigned w, int f) {
    const unsigned x = __shfl_sync(0xffffffffu, w, 12 + (f >> 2));
    return (int)(signed char)((x >> (8 * (f & 3))) & 0xffu);
  }
  static __device__ __forceinline__ int qd(unsigned w) { return (int)__shfl_sync(0xffffffffu, w, 14); }
  static __device__ __forceinline__ int tree(unsigned w) { return (int)__shfl_sync(0xffffffffu, w, 15); }
};

template <int D, int NC, class T, int W, int S, int ASYNC>
__global__ void __launch_bounds__(W * 32)
k_sweep_warp(Meta m, BoxSet bs, T* __restrict__ phi, const T* __restrict__ rhs, int n, int pull,
             int homog) {
  // Everything up to the first data-dependent load runs before pdl_wait():
  // barrier set-up, per-lane constants and the first descriptors (the slot
  // tables and descriptors never change after the forest is created).
  pdl_trigger();
  using C = WarpCfg<D, NC, T, W, S>;
  using G = Geo<D, NC>;
  static_assert(S >= 2, "at least two stages");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar[W][S];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)gridDim.x * W;
  const int nbx = bs.n;
  // few boxes (grid sized one block per box): spread them over the SMs
  const int gw = nbx <= nw ? wid * (int)gridDim.x + (int)blockIdx.x : (int)blockIdx.x * W + wid;
  if (gw >= nbx) {
    pdl_wait();
    return;
  }
  const int my_boxes = (nbx - 1 - gw) / nw + 1;
  unsigned char* ring = smem + (size_t)wid * S * C::BOX_B;
  if (lane == 0) {
    for (int st = 0; st < S; ++st) mbar_init(&bar[wid][st], 1);
    fence_mbar_init();
  }
  __syncwarp();

  // Per-lane constants: ghost items and updated cells.
  int it_f[C::GPL], it_gpos[C::GPL], it_npos[C::GPL], it_apos[C::GPL], it_lin[C::GPL];
  short it_gi[C::GPL], it_gj[C::GPL], it_gk[C::GPL];
  bool it_on[C::GPL];
#pragma unroll
  for (int j = 0; j < C::GPL; ++j) {
    const int r = lane + 32 * j;
    it_on[j] = r < C::NEED;
    const int rr = it_on[j] ? r : 0;
    const int f = rr / (G::NF / 2);
    int a, c;
    needed_face_cell<D, NC>(f, rr % (G::NF / 2), n, a, c);
    const Face<D, NC> F(f, a, c);
    it_f[j] = f;
    it_gpos[j] = G::g(F.gi, F.gj, F.gk);
    it_npos[j] = G::g(F.ni, F.nj, F.nk);
    it_apos[j] = G::g(F.ai, F.aj, F.ak);
    it_lin[j] = (D == 2) ? (a - 1) : (a - 1) + NC * (c - 1);
    it_gi[j] = (short)F.gi;
    it_gj[j] = (short)F.gj;
    it_gk[j] = (short)F.gk;
  }
  int upos[C::CPL], rpos[C::CPL];
  bool uon[C::CPL];
#pragma unroll
  for (int c = 0; c < C::CPL; ++c) {
    const int uq = lane + 32 * c;
    uon[c] = uq < C::UPD;
    const int q = uon[c] ? uq : 0;
    const int p = q % (NC / 2);
    if constexpr (D == 2) {
      const int j = q / (NC / 2) + 1;
      const int i = 2 * p + 1 + ((1 + j + n) & 1);
      upos[c] = G::g(i, j, 0);
      rpos[c] = G::in(i, j, 1);
    } else {
      const int j = (q / (NC / 2)) % NC + 1;
      const int k = q / ((NC / 2) * NC) + 1;
      const int i = 2 * p + 1 + ((1 + j + k + n) & 1);
      upos[c] = G::g(i, j, k);
      rpos[c] = G::in(i, j, k);
    }
  }
  constexpr int OX = 1, OY = G::NG, OZ = G::NG * G::NG;

  int issued = 0;  // boxes whose copies lane 0 has issued
  auto stage = [&](int k) { return ring + (k % S) * C::BOX_B; };
  auto issue = [&](int k) {  // lane 0 (bulk copies) or all lanes (cp.async)
    ++issued;
    const int i = gw + k * nw;
    const int s = box_at(bs, i);
    unsigned char* sp = stage(k);
    if constexpr (ASYNC) {
      const unsigned char* src = reinterpret_cast<const unsigned char*>(phi + box_offg<G::SG>(m, bs, i, s));
      for (int q = lane; q < (G::SG * (int)sizeof(T)) / 16; q += 32) cp_async16(sp + C::PHI_OFF + 16 * q, src + 16 * q);
      if (lane < (int)sizeof(SlotDesc) / 16)
        cp_async16(sp + 16 * lane, reinterpret_cast<const unsigned char*>(m.desc + s) + 16 * lane);
    } else {
      unsigned long long* b = &bar[wid][k % S];
      fence_proxy_async();
      mbar_expect_tx(b, (unsigned)C::BOX_B);
      bulk_g2s(sp, m.desc + s, (unsigned)sizeof(SlotDesc), b);
      bulk_g2s(sp + C::PHI_OFF, phi + box_offg<G::SG>(m, bs, i, s), (unsigned)(G::SG * sizeof(T)), b);
    }
  };
  // Descriptor words of box k, straight from global memory (the ghost
  // sources are fetched two boxes ahead, before the box's bulk copy lands).
  auto desc_words = [&](int k) -> unsigned {
    if (k >= my_boxes) return 0u;
    const int s = box_at(bs, gw + k * nw);
    return reinterpret_cast<const unsigned*>(m.desc + s)[lane];
  };
  // Ghost sources and rhs values of box k from its descriptor words.
  auto fetch = [&](int k, unsigned w, bool live, T (&val)[C::GPL], T (&rv)[C::CPL], int& act) {
    act = 0;
#pragma unroll
    for (int j = 0; j < C::GPL; ++j) val[j] = (T)0;
#pragma unroll
    for (int c = 0; c < C::CPL; ++c) rv[c] = (T)0;
    if (!live) return;
    act = m.active[DescWords::tree(w)];
    {
      const int i = gw + k * nw;
      const T* rb = rhs + box_offi<G::SI>(m, bs, i, bs.list ? bs.list[i] : 0);
#pragma unroll
      for (int c = 0; c < C::CPL; ++c)
        if (uon[c]) rv[c] = rb[rpos[c]];
    }
    const int qd = DescWords::qd(w);
#pragma unroll
    for (int j = 0; j < C::GPL; ++j) {
      const int f = it_f[j];
      const int code = DescWords::code(w, f);
      const long long o = DescWords::nbo(w, f);
      if (!pull || !it_on[j]) continue;
      if (code >= 0) {
        val[j] = phi[o + it_npos[j]];
      } else if (code == kFaceRefinement) {
        const int h = NC >> 1;
        const int pi = (qd & 1) * h + ((it_gi[j] + 1) >> 1);
        const int pj = ((qd >> 1) & 1) * h + ((it_gj[j] + 1) >> 1);
        const int pk = (D == 3) ? ((qd >> 2) & 1) * h + ((it_gk[j] + 1) >> 1) : 0;
        val[j] = phi[o + G::g(pi, pj, pk)];
      } else if (o >= 0 && !homog) {
        val[j] = (T)m.bcval[o + it_lin[j]];
      }
    }
  };
  // Box k: issue box k+S-1, read the descriptor of box k+4, fetch the ghost
  // sources of box k+2, then update box k from its stage with the ghost
  // sources fetched two boxes ago. False if a bounded wait gave up.
  auto body = [&](int k, T (&g0)[C::GPL], T (&r0)[C::CPL], int& a0, T (&g2)[C::GPL], T (&r2)[C::CPL],
                  int& a2, unsigned& w2, unsigned& w4) -> bool {
    if constexpr (ASYNC) {
      if (k + S - 1 < my_boxes) issue(k + S - 1);
      cp_async_commit();  // one group per box (empty past the end)
    } else {
      if (lane == 0 && k + S - 1 < my_boxes) issue(k + S - 1);
    }
    const unsigned w_new = desc_words(k + 4);
    fetch(k + 2, w2, k + 2 < my_boxes, g2, r2, a2);
    if constexpr (ASYNC) {
      cp_async_wait<S - 1>();  // box k's group has landed
      __syncwarp();
    } else {
      const bool ok = mbar_wait_bounded(&bar[wid][k % S], (k / S) & 1, m.wait_limit);
      if (!__all_sync(0xffffffffu, ok)) return false;
    }
    unsigned char* sp = stage(k);
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(sp);
    T* bx = reinterpret_cast<T*>(sp + C::PHI_OFF);
    if (a0) {
      if (pull) {
#pragma unroll
        for (int j = 0; j < C::GPL; ++j) {
          if (!it_on[j]) continue;
          const int f = it_f[j];
          const int code = d.code[f];
          T v = g0[j];
          if (code < 0) {
            if (code == kFaceRefinement) {  // mg$D_sides_rb, src/m_aX_mg.f90:286-347
              const int dix = (f & 1) ? -1 : 1;
              const int ap = it_apos[j];
              const int dim = f >> 1;
              if constexpr (D == 2) {
                if (dim == 0) {
                  const int dj = -1 + 2 * ((int)it_gj[j] & 1);
                  v = (T)0.5 * g0[j] + bx[ap] - (T)0.25 * (bx[ap + dix * OX] + bx[ap + dj * OY]);
                } else {
                  const int di = -1 + 2 * ((int)it_gi[j] & 1);
                  v = (T)0.5 * g0[j] + bx[ap] - (T)0.25 * (bx[ap + di * OX] + bx[ap + dix * OY]);
                }
              } else {
                const int ti = (int)it_gi[j], tj = (int)it_gj[j], tk = (int)it_gk[j];
                const int di = (dim == 0) ? dix : -1 + 2 * (ti & 1);
                const int dj = (dim == 1) ? dix : -1 + 2 * (tj & 1);
                const int dk = (dim == 2) ? dix : -1 + 2 * (tk & 1);
                v = (T)0.5 * g0[j] + (T)0.75 * bx[ap] - (T)0.25 * bx[ap + di * OX + dj * OY + dk * OZ];
              }
            } else {
              v = bc_value<T>(code, f, g0[j], bx[it_apos[j]], Sc<T>::dr(d));
            }
          }
          bx[it_gpos[j]] = v;
        }
        __syncwarp();
      }
      const T dx2 = Sc<T>::dx2(d);
      T* out = phi + d.offg;
#pragma unroll
      for (int c = 0; c < C::CPL; ++c) {
        if (!uon[c]) continue;
        const T* b = bx + upos[c];
        const T f = r0[c];
        T v;
        if constexpr (D == 2) {
          v = (T)0.25 * (b[OX] + b[-OX] + b[OY] + b[-OY] - dx2 * f);
        } else {
          const T sixth = (T)(1 / 6.0);
          v = sixth * (b[OX] + b[-OX] + b[OY] + b[-OY] + b[OZ] + b[-OZ] - dx2 * f);
        }
        out[upos[c]] = v;
      }
    }
    __syncwarp();  // the stage of box k is refilled at box k + 1
    w2 = w4;       // rotate: the words of box k+3 move up
    w4 = w_new;
    return true;
  };

  const unsigned w0 = desc_words(0), w1 = desc_words(1);
  // Descriptor words of boxes k+2 and k+3 at the start of box k.
  unsigned wq = desc_words(2), wr = desc_words(3);
  pdl_wait();  // the previous kernel's writes to phi are visible from here on
  if constexpr (ASYNC) {
    for (int k = 0; k < S - 1; ++k) {
      if (k < my_boxes) issue(k);
      cp_async_commit();
    }
  } else {
    if (lane == 0)
      for (int k = 0; k < S - 1 && k < my_boxes; ++k) issue(k);
  }
  T ga[C::GPL], gb[C::GPL], gc[C::GPL];
  T ra[C::CPL], rb[C::CPL], rc[C::CPL];
  int aa = 0, ab = 0, ac = 0;
  fetch(0, w0, true, ga, ra, aa);
  fetch(1, w1, 1 < my_boxes, gb, rb, ab);
  int k = 0;
  bool ok = true;
  for (; k < my_boxes; k += 3) {
    // body(k) uses set a and fetches box k+2 into set c; words rotate wq <- wr <- new
    if (!(ok = body(k, ga, ra, aa, gc, rc, ac, wq, wr))) break;
    if (k + 1 >= my_boxes) break;
    if (!(ok = body(k + 1, gb, rb, ab, ga, ra, aa, wq, wr))) { k += 1; break; }
    if (k + 2 >= my_boxes) break;
    if (!(ok = body(k + 2, gc, rc, ac, gb, rb, ab, wq, wr))) { k += 2; break; }
  }
  if constexpr (ASYNC) {
    cp_async_wait<0>();
  } else if (!ok && lane == 0) {  // gave up at box k: drain this warp's copies from box k on
    atomicExch(m.err, 1);
    for (int j = k; j < issued; ++j) mbar_wait_bounded(&bar[wid][j % S], (j / S) & 1, kDrainLimitCycles);
  }
}

// Laplacian of mg$D_box_lpl (src/m_aX_mg.f90:763-797) at (i,j,k) of a staged box.
template <int D, int NC, class T>
__device__ __forceinline__ T lpl_at(const T* bx, int i, int j, int k, T inv_dr_sq) {
  using G = Geo<D, NC>;
  if constexpr (D == 2) {
    return inv_dr_sq * (bx[G::g(i - 1, j, 0)] + bx[G::g(i + 1, j, 0)] + bx[G::g(i, j - 1, 0)] +
                        bx[G::g(i, j + 1, 0)] - (T)4 * bx[G::g(i, j, 0)]);
  } else {
    return inv_dr_sq * (bx[G::g(i - 1, j, k)] + bx[G::g(i + 1, j, k)] + bx[G::g(i, j - 1, k)] +
                        bx[G::g(i, j + 1, k)] + bx[G::g(i, j, k - 1)] + bx[G::g(i, j, k + 1)] -
                        (T)6 * bx[G::g(i, j, k)]);
  }
}

// ---------------------------------------------------------------------------
// Warp-per-box residual and restriction (the fine side of update_coarse,
// src/m_aX_mg.f90:424-451) on a level >= 2, with the ghost cells pulled: the
// pipeline of k_sweep_warp (bulk-copied box in an S-stage ring per warp),
// with every face ghost, the rhs of the lane's fine cells and the parent's
// offset fetched one box ahead. Each lane owns PPL parent cells and the 2^D
// fine cells of each; the residual and the restriction are summed in the
// order of k_restrict_res.
// ---------------------------------------------------------------------------
template <int D, int NC, class T, int W, int S>
struct RestrictCfg {
  using G = Geo<D, NC>;
  static constexpr int H = NC / 2;
  static constexpr int PAR = D == 2 ? H * H : H * H * H;  // parent cells per fine box
  static constexpr int PPL = (PAR + 31) / 32;             // per lane
  static constexpr int FINE = 1 << D;
  static constexpr int NEED = 2 * D * G::NF;              // every face ghost
  static constexpr int GPL = (NEED + 31) / 32;
  static constexpr int PHI_OFF = (int)sizeof(SlotDesc);
  static constexpr int BOX_B = PHI_OFF + G::SG * (int)sizeof(T);
  static constexpr int SMEM_B = W * S * BOX_B;
  static_assert(BOX_B % 16 == 0, "bulk copy alignment");
};

template <int D, int NC, class T, int W, int S>
__global__ void __launch_bounds__(W * 32)
k_restrict_warp(Meta m, BoxSet bs, T* __restrict__ phi, const T* __restrict__ rhs, T* __restrict__ tmp,
                int homog) {
  // Descriptors never change after the forest is created: those of the
  // first boxes are loaded before pdl_wait(), the cells after it.
  pdl_trigger();
  using C = RestrictCfg<D, NC, T, W, S>;
  using G = Geo<D, NC>;
  constexpr int H = C::H;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar[W][S];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)gridDim.x * W;
  const int nbx = bs.n;
  // few boxes (grid sized one block per box): spread them over the SMs
  const int gw = nbx <= nw ? wid * (int)gridDim.x + (int)blockIdx.x : (int)blockIdx.x * W + wid;
  if (gw >= nbx) {
    pdl_wait();
    return;
  }
  const int my_boxes = (nbx - 1 - gw) / nw + 1;
  unsigned char* ring = smem + (size_t)wid * S * C::BOX_B;
  if (lane == 0) {
    for (int st = 0; st < S; ++st) mbar_init(&bar[wid][st], 1);
    fence_mbar_init();
  }
  __syncwarp();

  int issued = 0;
  auto stage = [&](int k) { return ring + (k % S) * C::BOX_B; };
  auto issue = [&](int k) {  // lane 0
    ++issued;
    const int i = gw + k * nw;
    const int s = box_at(bs, i);
    unsigned char* sp = stage(k);
    unsigned long long* b = &bar[wid][k % S];
    fence_proxy_async();
    mbar_expect_tx(b, (unsigned)C::BOX_B);
    bulk_g2s(sp, m.desc + s, (unsigned)sizeof(SlotDesc), b);
    bulk_g2s(sp + C::PHI_OFF, phi + box_offg<G::SG>(m, bs, i, s), (unsigned)(G::SG * sizeof(T)), b);
  };
  auto issue_data = [&](int k) {  // lane 0: the cells only (descriptor staged)
    ++issued;
    const int i = gw + k * nw;
    const int s = box_at(bs, i);
    unsigned char* sp = stage(k);
    unsigned long long* b = &bar[wid][k % S];
    fence_proxy_async();
    mbar_expect_tx(b, (unsigned)(C::BOX_B - (int)sizeof(SlotDesc)));
    bulk_g2s(sp + C::PHI_OFF, phi + box_offg<G::SG>(m, bs, i, s), (unsigned)(G::SG * sizeof(T)), b);
  };
  // Item j of this lane: face f and face cell (a, c).
  auto item = [&](int j, int& f, int& a, int& c) {
    const int r = lane + 32 * j;
    f = r / G::NF;
    const int lin = r % G::NF;
    a = lin % NC + 1;
    c = lin / NC + 1;
  };
  // Ghost sources, rhs values and the parent's offset of box k (its
  // descriptor has landed).
  auto fetch = [&](int k, T (&gv)[C::GPL], T (&rv)[C::PPL][C::FINE], long long& po, int& act) {
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(stage(k));
    act = m.active[d.tree];
    po = m.offg[d.parent];
#pragma unroll
    for (int j = 0; j < C::GPL; ++j) {
      gv[j] = (T)0;
      if (lane + 32 * j >= C::NEED) continue;
      int f, a, c;
      item(j, f, a, c);
      const Face<D, NC> F(f, a, c);
      const int code = d.code[f];
      const long long o = d.nbo[f];
      if (code >= 0) {
        gv[j] = phi[o + G::g(F.ni, F.nj, F.nk)];
      } else if (code == kFaceRefinement) {
        gv[j] = phi[o + parent_cell<D, NC>(F, f, d.qd, false)];
      } else if (o >= 0 && !homog) {
        gv[j] = (T)m.bcval[o + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
      }
    }
    const T* f = rhs + d.offi;
#pragma unroll
    for (int p = 0; p < C::PPL; ++p) {
      const int q = lane + 32 * p;
      const int qq = q < C::PAR ? q : 0;
      const int ic = qq % H + 1, jc = (qq / H) % H + 1, kc = (D == 3) ? qq / (H * H) + 1 : 0;
      constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
      for (int kk = 0; kk < KK; ++kk)
#pragma unroll
        for (int jj = 0; jj < 2; ++jj)
#pragma unroll
          for (int ii = 0; ii < 2; ++ii)
            rv[p][(kk * 2 + jj) * 2 + ii] =
                f[G::in(2 * ic - 1 + ii, 2 * jc - 1 + jj, (D == 3) ? 2 * kc - 1 + kk : 1)];
    }
  };
  auto body = [&](int k, T (&g0)[C::GPL], T (&r0)[C::PPL][C::FINE], long long po0, int a0, T (&g1)[C::GPL],
                  T (&r1)[C::PPL][C::FINE], long long& po1, int& a1) -> bool {
    if (lane == 0 && k + S - 1 < my_boxes) issue(k + S - 1);
    bool ok = true;
    if (k + 1 < my_boxes) {
      ok = mbar_wait_bounded(&bar[wid][(k + 1) % S], ((k + 1) / S) & 1, m.wait_limit);
      if (ok) fetch(k + 1, g1, r1, po1, a1);
    }
    if (!__all_sync(0xffffffffu, ok)) return false;
    unsigned char* sp = stage(k);
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(sp);
    T* bx = reinterpret_cast<T*>(sp + C::PHI_OFF);
    if (a0) {
#pragma unroll
      for (int j = 0; j < C::GPL; ++j) {
        if (lane + 32 * j >= C::NEED) continue;
        int f, a, c;
        item(j, f, a, c);
        const Face<D, NC> F(f, a, c);
        const int code = d.code[f];
        T v = g0[j];
        if (code < 0) {
          auto own = [&](int i, int jj, int kk) { return bx[G::g(i, jj, kk)]; };
          if (code == kFaceRefinement)
            v = rb_value<D, NC, T>(F, f, g0[j], own);
          else
            v = bc_value<T>(code, f, g0[j], own(F.ai, F.aj, F.ak), Sc<T>::dr(d));
        }
        bx[G::g(F.gi, F.gj, F.gk)] = v;
      }
      __syncwarp();
      const T inv = Sc<T>::inv(d);
      const int qd = d.qd;
      const int off0 = (qd & 1) * H, off1 = ((qd >> 1) & 1) * H, off2 = ((qd >> 2) & 1) * H;
      using GP = Geo<D, NC>;
#pragma unroll
      for (int p = 0; p < C::PPL; ++p) {
        const int q = lane + 32 * p;
        if (q >= C::PAR) continue;
        const int ic = q % H + 1, jc = (q / H) % H + 1, kc = (D == 3) ? q / (H * H) + 1 : 0;
        T sr = 0, sp2 = 0;
        constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
        for (int kk = 0; kk < KK; ++kk)
#pragma unroll
          for (int jj = 0; jj < 2; ++jj)
#pragma unroll
            for (int ii = 0; ii < 2; ++ii) {
              const int i = 2 * ic - 1 + ii, j = 2 * jc - 1 + jj, kz = (D == 3) ? 2 * kc - 1 + kk : 0;
              const T r = r0[p][(kk * 2 + jj) * 2 + ii] - lpl_at<D, NC, T>(bx, i, j, kz, inv);
              sr = sr + r;
              sp2 = sp2 + bx[G::g(i, j, kz)];
            }
        const T w = (D == 2) ? (T)0.25 : (T)0.125;
        const long long o = po0 + GP::g(off0 + ic, off1 + jc, (D == 3) ? off2 + kc : 0);
        tmp[o] = w * sr;
        phi[o] = w * sp2;
      }
    }
    __syncwarp();  // the stage of box k is refilled at box k + 1
    return true;
  };

  const int ahead = min(S - 1, my_boxes);
  for (int k = 0; k < ahead; ++k)
    reinterpret_cast<unsigned*>(stage(k))[lane] =
        reinterpret_cast<const unsigned*>(m.desc + box_at(bs, gw + k * nw))[lane];
  __syncwarp();
  pdl_wait();  // the previous kernel's writes are visible from here on
  if (lane == 0)
    for (int k = 0; k < ahead; ++k) issue_data(k);
  T ga[C::GPL], gb[C::GPL];
  T ra[C::PPL][C::FINE], rb[C::PPL][C::FINE];
  long long pa = 0, pb = 0;
  int aa = 0, ab = 0;
  fetch(0, ga, ra, pa, aa);  // from the staged descriptor, beside the cells' copy
  bool ok = mbar_wait_bounded(&bar[wid][0], 0, m.wait_limit);
  int k = 0, pending = 0;
  if (__all_sync(0xffffffffu, ok)) {
    for (; k < my_boxes; k += 2) {
      if (!body(k, ga, ra, pa, aa, gb, rb, pb, ab)) break;
      if (k + 1 < my_boxes && !body(k + 1, gb, rb, pb, ab, ga, ra, pa, aa)) {
        k += 1;
        break;
      }
    }
    pending = k + 1;
  }
  if (k < my_boxes && lane == 0) {  // gave up: drain this warp's copies
    atomicExch(m.err, 1);
    for (int j = pending; j < issued; ++j) mbar_wait_bounded(&bar[wid][j % S], (j / S) & 1, kDrainLimitCycles);
  }
}

// ---------------------------------------------------------------------------
// Warp-per-box coarse right-hand side (the coarse side of update_coarse,
// src/m_aX_mg.f90:452-480) on a list of parents: the pipeline of
// k_restrict_warp; the pulled ghosts are stored (the reference's ghost fill
// of the coarse level), rhs = L phi + tmp on the interior, tmp = phi on the
// whole box. Each lane owns CPL interior cells; their tmp values are fetched
// one box ahead.
// ---------------------------------------------------------------------------
template <int D, int NC, class T, int W, int S>
struct CoarseCfg {
  using G = Geo<D, NC>;
  static constexpr int CPL = (G::SI + 31) / 32;
  static constexpr int NEED = 2 * D * G::NF;
  static constexpr int GPL = (NEED + 31) / 32;
  static constexpr int PHI_OFF = (int)sizeof(SlotDesc);
  static constexpr int BOX_B = PHI_OFF + G::SG * (int)sizeof(T);
  static constexpr int SMEM_B = W * S * BOX_B;
  static_assert(BOX_B % 16 == 0, "bulk copy alignment");
};

template <int D, int NC, class T, int W, int S>
__global__ void __launch_bounds__(W * 32)
k_coarse_warp(Meta m, BoxSet bs, T* __restrict__ phi, T* __restrict__ rhs, T* __restrict__ tmp, int homog) {
  // Descriptors never change after the forest is created: those of the
  // first boxes are loaded before pdl_wait(), the cells after it.
  pdl_trigger();
  using C = CoarseCfg<D, NC, T, W, S>;
  using G = Geo<D, NC>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar[W][S];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)gridDim.x * W;
  const int nbx = bs.n;
  // few boxes (grid sized one block per box): spread them over the SMs
  const int gw = nbx <= nw ? wid * (int)gridDim.x + (int)blockIdx.x : (int)blockIdx.x * W + wid;
  if (gw >= nbx) {
    pdl_wait();
    return;
  }
  const int my_boxes = (nbx - 1 - gw) / nw + 1;
  unsigned char* ring = smem + (size_t)wid * S * C::BOX_B;
  if (lane == 0) {
    for (int st = 0; st < S; ++st) mbar_init(&bar[wid][st], 1);
    fence_mbar_init();
  }
  __syncwarp();

  int issued = 0;
  auto stage = [&](int k) { return ring + (k % S) * C::BOX_B; };
  auto issue = [&](int k) {  // lane 0
    ++issued;
    const int i = gw + k * nw;
    const int s = box_at(bs, i);
    unsigned char* sp = stage(k);
    unsigned long long* b = &bar[wid][k % S];
    fence_proxy_async();
    mbar_expect_tx(b, (unsigned)C::BOX_B);
    bulk_g2s(sp, m.desc + s, (unsigned)sizeof(SlotDesc), b);
    bulk_g2s(sp + C::PHI_OFF, phi + box_offg<G::SG>(m, bs, i, s), (unsigned)(G::SG * sizeof(T)), b);
  };
  auto issue_data = [&](int k) {  // lane 0: the cells only (descriptor staged)
    ++issued;
    const int i = gw + k * nw;
    const int s = box_at(bs, i);
    unsigned char* sp = stage(k);
    unsigned long long* b = &bar[wid][k % S];
    fence_proxy_async();
    mbar_expect_tx(b, (unsigned)(C::BOX_B - (int)sizeof(SlotDesc)));
    bulk_g2s(sp + C::PHI_OFF, phi + box_offg<G::SG>(m, bs, i, s), (unsigned)(G::SG * sizeof(T)), b);
  };
  auto item = [&](int j, int& f, int& a, int& c) {
    const int r = lane + 32 * j;
    f = r / G::NF;
    const int lin = r % G::NF;
    a = lin % NC + 1;
    c = lin / NC + 1;
  };
  auto fetch = [&](int k, T (&gv)[C::GPL], T (&tv)[C::CPL], int& act) {
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(stage(k));
    act = m.active[d.tree];
#pragma unroll
    for (int j = 0; j < C::GPL; ++j) {
      gv[j] = (T)0;
      if (lane + 32 * j >= C::NEED) continue;
      int f, a, c;
      item(j, f, a, c);
      const Face<D, NC> F(f, a, c);
      const int code = d.code[f];
      const long long o = d.nbo[f];
      if (code >= 0) {
        gv[j] = phi[o + G::g(F.ni, F.nj, F.nk)];
      } else if (code == kFaceRefinement) {
        gv[j] = phi[o + parent_cell<D, NC>(F, f, d.qd, false)];
      } else if (o >= 0 && !homog) {
        gv[j] = (T)m.bcval[o + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
      }
    }
    const T* t = tmp + d.offg;
#pragma unroll
    for (int c = 0; c < C::CPL; ++c) {
      const int q = lane + 32 * c;
      const int qq = q < G::SI ? q : 0;
      const int i = qq % NC + 1, j = (qq / NC) % NC + 1, kz = (D == 3) ? qq / (NC * NC) + 1 : 0;
      tv[c] = t[G::g(i, j, kz)];
    }
  };
  auto body = [&](int k, T (&g0)[C::GPL], T (&t0)[C::CPL], int a0, T (&g1)[C::GPL], T (&t1)[C::CPL],
                  int& a1) -> bool {
    if (lane == 0 && k + S - 1 < my_boxes) issue(k + S - 1);
    bool ok = true;
    if (k + 1 < my_boxes) {
      ok = mbar_wait_bounded(&bar[wid][(k + 1) % S], ((k + 1) / S) & 1, m.wait_limit);
      if (ok) fetch(k + 1, g1, t1, a1);
    }
    if (!__all_sync(0xffffffffu, ok)) return false;
    unsigned char* sp = stage(k);
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(sp);
    T* bx = reinterpret_cast<T*>(sp + C::PHI_OFF);
    if (a0) {
      T* gphi = phi + d.offg;
#pragma unroll
      for (int j = 0; j < C::GPL; ++j) {
        if (lane + 32 * j >= C::NEED) continue;
        int f, a, c;
        item(j, f, a, c);
        const Face<D, NC> F(f, a, c);
        const int code = d.code[f];
        T v = g0[j];
        if (code < 0) {
          auto own = [&](int i, int jj, int kk) { return bx[G::g(i, jj, kk)]; };
          if (code == kFaceRefinement)
            v = rb_value<D, NC, T>(F, f, g0[j], own);
          else
            v = bc_value<T>(code, f, g0[j], own(F.ai, F.aj, F.ak), Sc<T>::dr(d));
        }
        const int gp = G::g(F.gi, F.gj, F.gk);
        bx[gp] = v;
        gphi[gp] = v;
      }
      __syncwarp();
      const T inv = Sc<T>::inv(d);
      T* r = rhs + d.offi;
#pragma unroll
      for (int c = 0; c < C::CPL; ++c) {
        const int q = lane + 32 * c;
        if (q >= G::SI) continue;
        const int i = q % NC + 1, j = (q / NC) % NC + 1, kz = (D == 3) ? q / (NC * NC) + 1 : 0;
        const T l = lpl_at<D, NC, T>(bx, i, j, kz, inv);
        r[q] = l + t0[c];
      }
      T* gt = tmp + d.offg;
      for (int e = lane; e < G::SG; e += 32) gt[e] = bx[e];
    }
    __syncwarp();  // the stage of box k is refilled at box k + 1
    return true;
  };

  const int ahead = min(S - 1, my_boxes);
  for (int k = 0; k < ahead; ++k)
    reinterpret_cast<unsigned*>(stage(k))[lane] =
        reinterpret_cast<const unsigned*>(m.desc + box_at(bs, gw + k * nw))[lane];
  __syncwarp();
  pdl_wait();  // the previous kernel's writes are visible from here on
  if (lane == 0)
    for (int k = 0; k < ahead; ++k) issue_data(k);
  T ga[C::GPL], gb[C::GPL], ta[C::CPL], tb[C::CPL];
  int aa = 0, ab = 0;
  fetch(0, ga, ta, aa);  // from the staged descriptor, beside the cells' copy
  bool ok = mbar_wait_bounded(&bar[wid][0], 0, m.wait_limit);
  int k = 0, pending = 0;
  if (__all_sync(0xffffffffu, ok)) {
    for (; k < my_boxes; k += 2) {
      if (!body(k, ga, ta, aa, gb, tb, ab)) break;
      if (k + 1 < my_boxes && !body(k + 1, gb, tb, ab, ga, ta, aa)) {
        k += 1;
        break;
      }
    }
    pending = k + 1;
  }
  if (k < my_boxes && lane == 0) {  // gave up: drain this warp's copies
    atomicExch(m.err, 1);
    for (int j = pending; j < issued; ++j) mbar_wait_bounded(&bar[wid][j % S], (j / S) & 1, kDrainLimitCycles);
  }
}

// ---------------------------------------------------------------------------
// Warp-per-parent correct_children (src/m_aX_mg.f90:368-395) for children on
// levels >= 2: the pipeline of k_restrict_warp on a list of parents, with the
// parent's tmp staged beside its phi. With pull the parent's face ghosts are
// recomputed and stored first (their sources fetched one parent ahead); then
// tmp = phi - tmp over the ghosted box (stored), and each lane adds the
// prolongation (mg$D_box_corr_lpl :708-715) of its parent cells to the 2^D
// fine cells each covers. The fine cells of P parent cells are loaded before
// any of them is stored, one batch ahead of the batch being stored, so that
// a lane keeps up to 2 P 2^D loads in flight. The children of a parent are
// consecutive slots of one level, stored SG apart.
// ---------------------------------------------------------------------------
template <int D, int NC, class T, int W, int S>
struct CorrectCfg {
  using G = Geo<D, NC>;
  static constexpr int H = NC / 2;
  static constexpr int FINE = 1 << D;
  static constexpr int CPL = (G::SI + 31) / 32;  // parent interior cells per lane
  static constexpr int NEED = 2 * D * G::NF;
  static constexpr int GPL = (NEED + 31) / 32;
  // parent cells per batch: 16 fine-cell loads in either precision
  static constexpr int PW = 16 / FINE;
  static constexpr int P = PW < CPL ? PW : CPL;
  static constexpr int NB = (CPL + P - 1) / P;
  static constexpr int PHI_OFF = (int)sizeof(SlotDesc);
  static constexpr int TMP_OFF = PHI_OFF + G::SG * (int)sizeof(T);
  static constexpr int BOX_B = TMP_OFF + G::SG * (int)sizeof(T);
  static constexpr int SMEM_B = W * S * BOX_B;
  static_assert(TMP_OFF % 16 == 0 && BOX_B % 16 == 0, "bulk copy alignment");
  static_assert(S >= 3, "sources are fetched one parent ahead of the one in use");
};

template <int D, int NC, class T, int W, int S, int SPLIT>
__global__ void __launch_bounds__(W * 32)
k_correct_warp(Meta m, BoxSet bs, T* __restrict__ phi, T* __restrict__ tmp, int pull, int homog) {
  constexpr int split = SPLIT;
  // Descriptors never change after the forest is created: those of the
  // first boxes are loaded before pdl_wait(), the cells after it.
  pdl_trigger();
  using C = CorrectCfg<D, NC, T, W, S>;
  using G = Geo<D, NC>;
  using V = typename Vec<T>::type;
  constexpr int VW = Vec<T>::w;
  constexpr int H = C::H, FINE = C::FINE, P = C::P;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar[W][S];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)gridDim.x * W;
  // split 0: one warp per parent does it all. For levels with few parents,
  // whose per-parent work would otherwise sit on one SM, two launches:
  // split 1, a warp per parent makes the ghosts and tmp = phi - tmp and
  // stores them; split 2, a warp per (parent, child) stages the stored tmp
  // and adds the prolongation of that child's quadrant.
  const int per = split == 2 ? C::FINE : 1;
  const int nbx = bs.n * per;
  // few items (grid sized one block per item): spread them over the SMs
  const int gw = nbx <= nw ? wid * (int)gridDim.x + (int)blockIdx.x : (int)blockIdx.x * W + wid;
  if (gw >= nbx) {
    pdl_wait();
    return;
  }
  const int my_boxes = (nbx - 1 - gw) / nw + 1;
  auto parent_of = [&](int k) { return (gw + k * nw) / per; };
  auto child_of = [&](int k) { return split == 2 ? (gw + k * nw) % per : -1; };
  unsigned char* ring = smem + (size_t)wid * S * C::BOX_B;
  if (lane == 0) {
    for (int st = 0; st < S; ++st) mbar_init(&bar[wid][st], 1);
    fence_mbar_init();
  }
  __syncwarp();

  int issued = 0;
  auto stage = [&](int k) { return ring + (k % S) * C::BOX_B; };
  auto issue = [&](int k) {  // lane 0
    ++issued;
    const int i = parent_of(k);
    const int s = box_at(bs, i);
    const long long o = box_offg<G::SG>(m, bs, i, s);
    unsigned char* sp = stage(k);
    unsigned long long* b = &bar[wid][k % S];
    fence_proxy_async();
    mbar_expect_tx(b, (unsigned)C::BOX_B);
    bulk_g2s(sp, m.desc + s, (unsigned)sizeof(SlotDesc), b);
    bulk_g2s(sp + C::PHI_OFF, phi + o, (unsigned)(G::SG * sizeof(T)), b);
    bulk_g2s(sp + C::TMP_OFF, tmp + o, (unsigned)(G::SG * sizeof(T)), b);
  };
  auto issue_data = [&](int k) {  // lane 0: the cells only (descriptor staged)
    ++issued;
    const int i = parent_of(k);
    const int s = box_at(bs, i);
    const long long o = box_offg<G::SG>(m, bs, i, s);
    unsigned char* sp = stage(k);
    unsigned long long* b = &bar[wid][k % S];
    fence_proxy_async();
    mbar_expect_tx(b, (unsigned)(C::BOX_B - (int)sizeof(SlotDesc)));
    bulk_g2s(sp + C::PHI_OFF, phi + o, (unsigned)(G::SG * sizeof(T)), b);
    bulk_g2s(sp + C::TMP_OFF, tmp + o, (unsigned)(G::SG * sizeof(T)), b);
  };
  auto item = [&](int j, int& f, int& a, int& c) {
    const int r = lane + 32 * j;
    f = r / G::NF;
    const int lin = r % G::NF;
    a = lin % NC + 1;
    c = lin / NC + 1;
  };
  // Activity, ghost sources (with pull) and the first child's offset of
  // parent k (its descriptor has landed).
  auto fetch = [&](int k, T (&gv)[C::GPL], long long& co, int& act) {
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(stage(k));
    act = m.active[d.tree];
    co = m.offg[d.first_child];
#pragma unroll
    for (int j = 0; j < C::GPL; ++j) {
      gv[j] = (T)0;
      if (!pull || split == 2 || lane + 32 * j >= C::NEED) continue;
      int f, a, c;
      item(j, f, a, c);
      const Face<D, NC> F(f, a, c);
      const int code = d.code[f];
      const long long o = d.nbo[f];
      if (code >= 0) {
        gv[j] = phi[o + G::g(F.ni, F.nj, F.nk)];
      } else if (code == kFaceRefinement) {
        gv[j] = phi[o + parent_cell<D, NC>(F, f, d.qd, false)];
      } else if (o >= 0 && !homog) {
        gv[j] = (T)m.bcval[o + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
      }
    }
  };
  // Offset (from the first child) of the first fine cell of parent cell q;
  // fine cell f of it is foff(f) further.
  auto fine_base = [&](int q) -> int {
    const int ic = q % NC + 1, jc = (q / NC) % NC + 1, kc = (D == 3) ? q / (NC * NC) + 1 : 0;
    const int qx = (ic - 1) / H, qy = (jc - 1) / H, qz = (D == 3) ? (kc - 1) / H : 0;
    const int li = ic - qx * H, lj = jc - qy * H, lk = (D == 3) ? kc - qz * H : 0;
    return (qx + 2 * qy + 4 * qz) * G::SG + G::g(2 * li - 1, 2 * lj - 1, (D == 3) ? 2 * lk - 1 : 0);
  };
  auto foff = [](int f) { return (f & 1) + ((f >> 1) & 1) * G::NG + ((f >> 2) & 1) * G::NG * G::NG; };
  // Parent cell (interior index) of this lane's item idx: all cells, or the
  // quadrant of child ch; false past the end.
  auto pcell = [&](int idx, int ch, int& q) -> bool {
    if (ch < 0) {
      q = lane + 32 * idx;
      return idx < C::CPL && q < G::SI;
    }
    const int lq = lane + 32 * idx;
    constexpr int QN = D == 2 ? H * H : H * H * H;
    if (lq >= QN) return false;
    const int li = lq % H, lj = (lq / H) % H, lk = (D == 3) ? lq / (H * H) : 0;
    q = ((ch & 1) * H + li) + NC * (((ch >> 1) & 1) * H + lj) +
        ((D == 3) ? NC * NC * (((ch >> 2) & 1) * H + lk) : 0);
    return true;
  };
  auto load_batch = [&](int nb, int ch, const T* cp, T (&buf)[P][FINE]) {
#pragma unroll
    for (int pp = 0; pp < P; ++pp) {
      int q;
      if (!pcell(nb * P + pp, ch, q)) continue;
      const T* c = cp + fine_base(q);
#pragma unroll
      for (int f = 0; f < FINE; ++f) buf[pp][f] = c[foff(f)];
    }
  };
  // phi(fine) = prolongation + old value, in the order of k_correct.
  auto store_batch = [&](int nb, int ch, T* cp, const T* t, const T (&buf)[P][FINE]) {
#pragma unroll
    for (int pp = 0; pp < P; ++pp) {
      int q;
      if (!pcell(nb * P + pp, ch, q)) continue;
      const int ic = q % NC + 1, jc = (q / NC) % NC + 1, kc = (D == 3) ? q / (NC * NC) + 1 : 0;
      const T f0 = t[G::g(ic, jc, kc)];
      const T fx = (T)0.125 * (t[G::g(ic + 1, jc, kc)] - t[G::g(ic - 1, jc, kc)]);
      const T fy = (T)0.125 * (t[G::g(ic, jc + 1, kc)] - t[G::g(ic, jc - 1, kc)]);
      const T fxx = (T)0.03125 * (t[G::g(ic - 1, jc, kc)] - (T)2 * f0 + t[G::g(ic + 1, jc, kc)]);
      const T fyy = (T)0.03125 * (t[G::g(ic, jc - 1, kc)] - (T)2 * f0 + t[G::g(ic, jc + 1, kc)]);
      T fz = 0, f2;
      if constexpr (D == 2) {
        f2 = fxx + fyy;
      } else {
        fz = (T)0.125 * (t[G::g(ic, jc, kc + 1)] - t[G::g(ic, jc, kc - 1)]);
        const T fzz = (T)0.03125 * (t[G::g(ic, jc, kc - 1)] - (T)2 * f0 + t[G::g(ic, jc, kc + 1)]);
        f2 = fxx + fyy + fzz;
      }
      T* c = cp + fine_base(q);
#pragma unroll
      for (int f = 0; f < FINE; ++f) {
        T v = f0;
        v = (f & 1) ? v + fx : v - fx;
        v = (f & 2) ? v + fy : v - fy;
        if constexpr (D == 3) v = (f & 4) ? v + fz : v - fz;
        c[foff(f)] = v + f2 + buf[pp][f];
      }
    }
  };
  auto body = [&](int k, T (&g0)[C::GPL], long long co0, int a0, T (&g1)[C::GPL], long long& co1,
                  int& a1) -> bool {
    if (lane == 0 && k + S - 1 < my_boxes) issue(k + S - 1);
    bool ok = true;
    if (k + 1 < my_boxes) {
      ok = mbar_wait_bounded(&bar[wid][(k + 1) % S], ((k + 1) / S) & 1, m.wait_limit);
      if (ok) fetch(k + 1, g1, co1, a1);
    }
    if (!__all_sync(0xffffffffu, ok)) return false;
    unsigned char* sp = stage(k);
    const SlotDesc& d = *reinterpret_cast<const SlotDesc*>(sp);
    T* bx = reinterpret_cast<T*>(sp + C::PHI_OFF);
    T* tx = reinterpret_cast<T*>(sp + C::TMP_OFF);
    if (a0) {
      const int ch = child_of(k);
      T ca[P][FINE], cb[P][FINE];
      T* cp = phi + co0;
      if (split != 1) load_batch(0, ch, cp, ca);  // the children's cells are not written before the stores below
      if (pull && split != 2) {
        T* gphi = phi + d.offg;
#pragma unroll
        for (int j = 0; j < C::GPL; ++j) {
          if (lane + 32 * j >= C::NEED) continue;
          int f, a, c;
          item(j, f, a, c);
          const Face<D, NC> F(f, a, c);
          const int code = d.code[f];
          T v = g0[j];
          if (code < 0) {
            auto own = [&](int i, int jj, int kk) { return bx[G::g(i, jj, kk)]; };
            if (code == kFaceRefinement)
              v = rb_value<D, NC, T>(F, f, g0[j], own);
            else
              v = bc_value<T>(code, f, g0[j], own(F.ai, F.aj, F.ak), Sc<T>::dr(d));
          }
          const int gp = G::g(F.gi, F.gj, F.gk);
          bx[gp] = v;
          gphi[gp] = v;
        }
        __syncwarp();
      }
      V* gt = reinterpret_cast<V*>(tmp + d.offg);
      for (int e = lane; split != 2 && e < G::SG / VW; e += 32) {
        const V p = reinterpret_cast<const V*>(bx)[e];
        const V t = reinterpret_cast<const V*>(tx)[e];
        V r;
        if constexpr (VW == 2) {
          r.x = p.x - t.x;
          r.y = p.y - t.y;
        } else {
          r.x = p.x - t.x;
          r.y = p.y - t.y;
          r.z = p.z - t.z;
          r.w = p.w - t.w;
        }
        reinterpret_cast<V*>(tx)[e] = r;
        gt[e] = r;
      }
      __syncwarp();
#pragma unroll
      for (int nb = 0; split != 1 && nb < C::NB; nb += 2) {
        if (nb + 1 < C::NB) load_batch(nb + 1, ch, cp, cb);
        store_batch(nb, ch, cp, tx, ca);
        if (nb + 1 < C::NB) {
          if (nb + 2 < C::NB) load_batch(nb + 2, ch, cp, ca);
          store_batch(nb + 1, ch, cp, tx, cb);
        }
      }
    }
    __syncwarp();  // the stage of parent k is refilled at parent k + 1
    return true;
  };

  const int ahead = min(S - 1, my_boxes);
  for (int k = 0; k < ahead; ++k)
    reinterpret_cast<unsigned*>(stage(k))[lane] =
        reinterpret_cast<const unsigned*>(m.desc + box_at(bs, parent_of(k)))[lane];
  __syncwarp();
  pdl_wait();  // the previous kernel's writes are visible from here on
  if (lane == 0)
    for (int k = 0; k < ahead; ++k) issue_data(k);
  T ga[C::GPL], gb[C::GPL];
  long long oa = 0, ob = 0;
  int aa = 0, ab = 0;
  fetch(0, ga, oa, aa);  // from the staged descriptor, beside the cells' copy
  bool ok = mbar_wait_bounded(&bar[wid][0], 0, m.wait_limit);
  int k = 0, pending = 0;
  if (__all_sync(0xffffffffu, ok)) {
    for (; k < my_boxes; k += 2) {
      if (!body(k, ga, oa, aa, gb, ob, ab)) break;
      if (k + 1 < my_boxes && !body(k + 1, gb, ob, ab, ga, oa, aa)) {
        k += 1;
        break;
      }
    }
    pending = k + 1;
  }
  if (k < my_boxes && lane == 0) {  // gave up: drain this warp's copies
    atomicExch(m.err, 1);
    for (int j = pending; j < issued; ++j) mbar_wait_bounded(&bar[wid][j % S], (j / S) & 1, kDrainLimitCycles);
  }
}

// ---------------------------------------------------------------------------
// Consecutive half-sweeps of a small level in one block (levels of at most a
// few boxes, where every half-sweep launched alone costs its launch and an L2
// round trip for little work). All boxes of the level and their rhs are
// loaded into shared memory once; each half-sweep first fills the ghost cells
// its colour reads from the current state (same-level neighbours from shared
// memory, coarse neighbours from the parent level, which does not change
// while the level is smoothed, and boundary values), then updates its colour
// in place; after the last one the interiors are written back. The values
// are those of the half-sweeps launched one by one (with pulled ghosts).
// ---------------------------------------------------------------------------
constexpr int kSmallThreads = 512;

template <int D, int NC, class T>
__global__ void __launch_bounds__(kSmallThreads)
k_sweep_small(Meta m, BoxSet bs, T* __restrict__ phi, const T* __restrict__ rhs, int n_first, int n_count,
              int pull_first, int homog) {
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int ITEMS = G::NNB * G::NF;  // face cells of a box
  extern __shared__ __align__(128) unsigned char smem[];
  const int nb = bs.n;
  SlotDesc* sd = reinterpret_cast<SlotDesc*>(smem);                   // nb descriptors
  T* sb = reinterpret_cast<T*>(smem + (size_t)nb * sizeof(SlotDesc));  // nb ghosted boxes
  T* sr = sb + (size_t)nb * G::SG;                                     // nb rhs interiors
  T* sc = sr + (size_t)nb * G::SI;                                     // per face cell: coarse value or boundary value
  int* sa = reinterpret_cast<int*>(sc + (size_t)nb * ITEMS);           // nb activity flags
  int* snb = sa + nb;  // per box and face: the same-level neighbour's index in the level, or -1
  constexpr int OX = 1, OY = G::NG, OZ = G::NG * G::NG;
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(m.desc + bs.lo);
    unsigned* dst = reinterpret_cast<unsigned*>(sd);
    for (int e = threadIdx.x; e < nb * (int)(sizeof(SlotDesc) / 4); e += blockDim.x) dst[e] = src[e];
  }
  pdl_wait();  // descriptors never change; phi, rhs and the flags may have been written by the previous kernel
  for (int e = threadIdx.x; e < nb * G::SG; e += blockDim.x) sb[e] = phi[bs.g0 + e];
  for (int e = threadIdx.x; e < nb * G::SI; e += blockDim.x) sr[e] = rhs[bs.i0 + e];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sa[b] = m.active[m.tree[bs.lo + b]];
  __syncthreads();
  for (int e = threadIdx.x; e < nb * G::NNB; e += blockDim.x) {
    const SlotDesc& d = sd[e / G::NNB];
    const int f = e % G::NNB;
    snb[e] = d.code[f] >= 0 ? (int)((d.nbo[f] - bs.g0) / G::SG) : -1;  // the neighbour is on this level
  }
  // The sources of the ghost cells that do not change while the level is
  // smoothed: the parent's injected cell at refinement boundaries, the
  // boundary value at physical faces.
  for (int e = threadIdx.x; e < nb * ITEMS; e += blockDim.x) {
    const int b = e / ITEMS, r = e % ITEMS;
    const int f = r / G::NF, lin = r % G::NF;
    const int a = lin % NC + 1, c = lin / NC + 1;
    const SlotDesc& d = sd[b];
    const int code = d.code[f];
    const long long o = d.nbo[f];
    T v = 0;
    if (code == kFaceRefinement) {
      v = phi[o + parent_cell<D, NC>(Face<D, NC>(f, a, c), f, d.qd, false)];
    } else if (code < 0 && !homog && o >= 0) {
      v = (T)m.bcval[o + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
    }
    sc[e] = v;
  }
  __syncthreads();
  for (int h = 0; h < n_count; ++h) {
    const int nsw = n_first + h;
    if (h > 0 || pull_first) {
      // only the ghost cells this colour reads: NF / 2 per face
      constexpr int HF = G::NF / 2;
      for (int e = threadIdx.x; e < nb * G::NNB * HF; e += blockDim.x) {
        const int pair = e / HF, mcell = e % HF;
        const int b = pair / G::NNB, f = pair % G::NNB;
        if (!sa[b]) continue;
        int a, c;
        needed_face_cell<D, NC>(f, mcell, nsw, a, c);
        const Face<D, NC> F(f, a, c);
        const SlotDesc& d = sd[b];
        T* bx = sb + (size_t)b * G::SG;
        const int code = d.code[f];
        T v;
        if (code >= 0) {
          v = sb[(size_t)snb[pair] * G::SG + G::g(F.ni, F.nj, F.nk)];
        } else {
          const T src = sc[(size_t)b * ITEMS + f * G::NF + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
          auto own = [&](int i, int j, int kk) { return bx[G::g(i, j, kk)]; };
          if (code == kFaceRefinement)
            v = rb_value<D, NC, T>(F, f, src, own);
          else
            v = bc_value<T>(code, f, src, own(F.ai, F.aj, F.ak), Sc<T>::dr(d));
        }
        bx[G::g(F.gi, F.gj, F.gk)] = v;
      }
      __syncthreads();
    }
    constexpr int HALF = G::SI / 2;
    for (int e = threadIdx.x; e < nb * HALF; e += blockDim.x) {
      const int b = e / HALF, q = e % HALF;
      if (!sa[b]) continue;
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
      T* bx = sb + (size_t)b * G::SG + upos;
      const T f = sr[(size_t)b * G::SI + rpos];
      const T dx2 = Sc<T>::dx2(sd[b]);
      T v;
      if constexpr (D == 2) {
        v = (T)0.25 * (bx[OX] + bx[-OX] + bx[OY] + bx[-OY] - dx2 * f);
      } else {
        const T sixth = (T)(1 / 6.0);
        v = sixth * (bx[OX] + bx[-OX] + bx[OY] + bx[-OY] + bx[OZ] + bx[-OZ] - dx2 * f);
      }
      *bx = v;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nb * G::SI; e += blockDim.x) {
    const int b = e / G::SI, q = e % G::SI;
    const int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
    const int gp = G::g(i, j, k);
    phi[bs.g0 + (long long)b * G::SG + gp] = sb[(size_t)b * G::SG + gp];
  }
}

// ---------------------------------------------------------------------------
// Half-sweep of a small level with one thread per updated cell and no
// staging (k_sweep_direct): on a level of a few dozen boxes the staged and
// pipelined sweeps are bound by their chain of dependent copies, not by
// bytes. Each thread reads its cell's neighbours straight from global memory;
// a neighbour across the box face is the ghost value this colour reads, made
// from the current state exactly as a pulled ghost (ghost_value): it depends
// on the cell itself (read before it is written, by the same thread) and on
// cells of the other colour, which no thread writes in this half-sweep. So
// the values are those of k_sweep_small and the staged sweeps, bit for bit.
// Without pull the stored ghost cells are read.
// ---------------------------------------------------------------------------
template <int D, int NC, class T>
__global__ void __launch_bounds__(kThreads)
k_sweep_direct(Meta m, BoxSet bs, T* phi, const T* rhs, int nsw, int pull, int homog) {
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int HALF = G::SI / 2;
  // one item per thread (the launch covers the level); the slot's tree and
  // descriptor never change, so they are read before the previous kernel ends
  const long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool mine = x < (long long)bs.n * HALF;
  const int b = mine ? (int)(x / HALF) : 0, q = mine ? (int)(x % HALF) : 0;
  const int s = mine ? box_at(bs, b) : 0;
  const int tr = mine ? m.tree[s] : 0;
  SlotDesc d;
  if (mine) d = m.desc[s];
  pdl_wait();
  if (!mine || !m.active[tr]) return;
  const int p = q % (NC / 2);
  int i, j, k;
  if constexpr (D == 2) {
    j = q / (NC / 2) + 1;
    k = 0;
    i = 2 * p + 1 + ((1 + j + nsw) & 1);
  } else {
    j = (q / (NC / 2)) % NC + 1;
    k = q / ((NC / 2) * NC) + 1;
    i = 2 * p + 1 + ((1 + j + k + nsw) & 1);
  }
  T* u = phi + d.offg;
  auto own = [&](int a, int bb, int c) { return u[G::g(a, bb, c)]; };
  // the neighbour of (i, j, k) in direction e (0: +x, 1: -x, 2: +y, 3: -y, 4: +z, 5: -z)
  auto nbv = [&](int e) -> T {
    const int dim = e >> 1, up = (e & 1) == 0;
    int c3[3] = {i, j, k};
    c3[dim] += up ? 1 : -1;
    const int x0 = c3[dim];
    if (x0 >= 1 && x0 <= NC) return u[G::g(c3[0], c3[1], c3[2])];
    if (!pull) return u[G::g(c3[0], c3[1], c3[2])];
    const int f = 2 * dim + (up ? 1 : 0);
    const int a = dim == 0 ? j : i, c = dim == 2 ? j : k;
    return ghost_value<D, NC, T>(m, d, phi, f, a, c, homog != 0, own);
  };
  const T f = rhs[d.offi + G::in(i, j, D == 3 ? k : 1)];
  const T dx2 = Sc<T>::dx2(d);
  T v;
  if constexpr (D == 2) {
    v = (T)0.25 * (nbv(0) + nbv(1) + nbv(2) + nbv(3) - dx2 * f);
  } else {
    const T sixth = (T)(1 / 6.0);
    v = sixth * (nbv(0) + nbv(1) + nbv(2) + nbv(3) + nbv(4) + nbv(5) - dx2 * f);
  }
  u[G::g(i, j, k)] = v;
}

// Loads a group of BPC boxes of a set into shared memory (whole ghosted
// boxes, vectorised) and their slots into s_slot; returns the count.
template <int D, int NC, class T, int BPC>
__device__ __forceinline__ int stage_boxes(const Meta& m, const BoxSet& bs, int grp, const T* __restrict__ src,
                                           T* sm, int* s_slot, int* s_act) {
  using G = Geo<D, NC>;
  using V = typename Vec<T>::type;
  constexpr int VW = Vec<T>::w;
  const int nbox = min(BPC, bs.n - grp * BPC);
  if ((int)threadIdx.x < BPC) {
    int s = (int)threadIdx.x < nbox ? box_at(bs, grp * BPC + threadIdx.x) : -1;
    s_slot[threadIdx.x] = s;
    s_act[threadIdx.x] = (s >= 0) ? m.active[m.tree[s]] : 0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nbox * (G::SG / VW); e += blockDim.x) {
    int b = e / (G::SG / VW), q = e % (G::SG / VW);
    reinterpret_cast<V*>(sm + b * G::SG)[q] = reinterpret_cast<const V*>(src + m.offg[s_slot[b]])[q];
  }
  __syncthreads();
  return nbox;
}

// Fills all face ghosts of the staged boxes from the level's current state.
template <int D, int NC, class T>
__device__ __forceinline__ void pull_all_ghosts(const Meta& m, const T* __restrict__ phi, T* sm,
                                                const int* s_slot, const int* s_act, int nbox, bool homog,
                                                T* store_to) {
  using G = Geo<D, NC>;
  for (int e = threadIdx.x; e < nbox * G::NNB * G::NF; e += blockDim.x) {
    const int b = e / (G::NNB * G::NF);
    const int r = e % (G::NNB * G::NF);
    const int f = r / G::NF, lin = r % G::NF;
    const int a = lin % NC + 1, c = lin / NC + 1;
    if (!s_act[b]) continue;
    const SlotDesc& d = m.desc[s_slot[b]];
    const T* bx = sm + b * G::SG;
    auto own = [&](int i, int j, int k) { return bx[G::g(i, j, k)]; };
    const T v = ghost_value<D, NC, T>(m, d, phi, f, a, c, homog, own);
    const Face<D, NC> F(f, a, c);
    const int gpos = G::g(F.gi, F.gj, F.gk);
    sm[b * G::SG + gpos] = v;
    if (store_to) store_to[d.offg + gpos] = v;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Residual and restriction to the parent: the per-box body of update_coarse
// and set_coarse_phi_rhs (src/m_aX_mg.f90:444-465, :495-504): residual_box
// (:545-559) then a$D_restrict_box of tmp and phi (src/m_aX_restrict.f90:67-132).
// The residual is kept in registers; the fine box's tmp is not written, which
// is what the reference's save/restore of tmp leaves behind (:452-462).
// SUB = the fine level is <= 1 (the parent is a sub-level box of half the size
// covering the same region, src/m_aX_t.f90:366-373). With pull the fine
// level's ghosts are recomputed here (no block writes that level).
// ---------------------------------------------------------------------------
template <int D, int NC, bool SUB, class T>
__global__ void __launch_bounds__(kThreads)
k_restrict_res(Meta m, BoxSet bs, T* __restrict__ phi, const T* __restrict__ rhs,
               T* __restrict__ tmp, int with_res, int pull, int homog) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int H = NC / 2;
  constexpr int PNC = SUB ? NC / 2 : NC;
  using GP = Geo<D, PNC>;
  constexpr int PER_BOX = D == 2 ? H * H : H * H * H;
  constexpr int BPC = boxes_per_cta<G::SG, PER_BOX, T>(1);
  __shared__ __align__(16) T sm[BPC * G::SG];
  __shared__ int s_slot[BPC];
  __shared__ int s_act[BPC];
  const int groups = (bs.n + BPC - 1) / BPC;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    const int nbox = stage_boxes<D, NC, T, BPC>(m, bs, grp, phi, sm, s_slot, s_act);
    if (pull && with_res) pull_all_ghosts<D, NC, T>(m, phi, sm, s_slot, s_act, nbox, homog != 0, nullptr);
    int b = threadIdx.x / PER_BOX, q = threadIdx.x % PER_BOX;
    if (b < nbox && s_act[b]) {
      int s = s_slot[b];
      const SlotDesc& d = m.desc[s];
      const T* bx = sm + b * G::SG;
      const T* f = rhs + d.offi;
      const T inv = Sc<T>::inv(d);
      int ic = q % H + 1, jc = (q / H) % H + 1, kc = (D == 3) ? q / (H * H) + 1 : 0;
      int off[3] = {0, 0, 0};
      if (!SUB) {
        const int qd = d.qd;
        off[0] = (qd & 1) * H;
        off[1] = ((qd >> 1) & 1) * H;
        off[2] = ((qd >> 2) & 1) * H;
      }
      T sr = 0, sp = 0;
      constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
      for (int kk = 0; kk < KK; ++kk)
#pragma unroll
        for (int jj = 0; jj < 2; ++jj)
#pragma unroll
          for (int ii = 0; ii < 2; ++ii) {
            int i = 2 * ic - 1 + ii, j = 2 * jc - 1 + jj, k = (D == 3) ? 2 * kc - 1 + kk : 0;
            if (with_res) {
              T r = f[G::in(i, j, k)] - lpl_at<D, NC, T>(bx, i, j, k, inv);
              sr = sr + r;
            }
            sp = sp + bx[G::g(i, j, k)];
          }
      const T w = (D == 2) ? (T)0.25 : (T)0.125;
      long long po = m.offg[d.parent] + GP::g(off[0] + ic, off[1] + jc, (D == 3) ? off[2] + kc : 0);
      if (with_res) tmp[po] = w * sr;
      phi[po] = w * sp;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Restriction of phi alone into the parents (a$D_restrict_box,
// src/m_aX_restrict.f90:67-132, as k_restrict_res without the residual): one
// thread per parent cell, its 2^D fine cells read straight from global
// memory in k_restrict_res's order. No ghost cell is read, so nothing is
// staged.
// ---------------------------------------------------------------------------
template <int D, int NC, bool SUB, class T>
__global__ void __launch_bounds__(kThreads)
k_restrict_phi(Meta m, BoxSet bs, T* __restrict__ phi) {
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int H = NC / 2;
  constexpr int PNC = SUB ? NC / 2 : NC;
  using GP = Geo<D, PNC>;
  constexpr int PAR = D == 2 ? H * H : H * H * H;
  pdl_wait();
  const long long total = (long long)bs.n * PAR;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int bi = (int)(x / PAR), q = (int)(x % PAR);
    const int s = box_at(bs, bi);
    if (!m.active[m.tree[s]]) continue;
    const T* bx = phi + box_offg<G::SG>(m, bs, bi, s);
    const int ic = q % H + 1, jc = (q / H) % H + 1, kc = (D == 3) ? q / (H * H) + 1 : 0;
    int off0 = 0, off1 = 0, off2 = 0;
    if (!SUB) {
      const int qd = m.desc[s].qd;
      off0 = (qd & 1) * H;
      off1 = ((qd >> 1) & 1) * H;
      off2 = ((qd >> 2) & 1) * H;
    }
    T sp = 0;
    constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
    for (int kk = 0; kk < KK; ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
          sp = sp + bx[G::g(2 * ic - 1 + ii, 2 * jc - 1 + jj, (D == 3) ? 2 * kc - 1 + kk : 0)];
    const T w = (D == 2) ? (T)0.25 : (T)0.125;
    phi[m.offg[m.parent[s]] + GP::g(off0 + ic, off1 + jc, (D == 3) ? off2 + kc : 0)] = w * sp;
  }
}

// ---------------------------------------------------------------------------
// Coarse right-hand side on the parents of a level after restriction
// (src/m_aX_mg.f90:472-479 and :510-515): rhs = L(phi) + tmp over the interior,
// then, for update_coarse, tmp = phi over the whole box including its ghosts
// (a$D_box_copy_cc, src/m_aX_utils.f90:331-339). With pull the parents'
// ghosts (fill_gc_phi of the parent level, :467) are recomputed here and
// stored.
// ---------------------------------------------------------------------------
template <int D, int NC, class T>
__global__ void __launch_bounds__(kThreads)
k_coarse_rhs(Meta m, BoxSet bs, T* __restrict__ phi, T* __restrict__ rhs,
             T* __restrict__ tmp, int copy_tmp, int pull, int homog) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int PER_BOX = G::SI < kThreads ? G::SI : kThreads;
  constexpr int BPC = boxes_per_cta<G::SG, PER_BOX, T>(1);
  using V = typename Vec<T>::type;
  constexpr int VW = Vec<T>::w;
  __shared__ __align__(16) T sm[BPC * G::SG];
  __shared__ int s_slot[BPC];
  __shared__ int s_act[BPC];
  const int groups = (bs.n + BPC - 1) / BPC;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    const int nbox = stage_boxes<D, NC, T, BPC>(m, bs, grp, phi, sm, s_slot, s_act);
    if (pull) pull_all_ghosts<D, NC, T>(m, phi, sm, s_slot, s_act, nbox, homog != 0, phi);
    int b = threadIdx.x / PER_BOX, q0 = threadIdx.x % PER_BOX;
    if (b < nbox && s_act[b]) {
      const SlotDesc& d = m.desc[s_slot[b]];
      const T* bx = sm + b * G::SG;
      const T inv = Sc<T>::inv(d);
      for (int q = q0; q < G::SI; q += PER_BOX) {
        int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
        T l = lpl_at<D, NC, T>(bx, i, j, k, inv);
        rhs[d.offi + q] = l + tmp[d.offg + G::g(i, j, k)];
      }
    }
    __syncthreads();
    if (copy_tmp) {
      for (int e = threadIdx.x; e < nbox * (G::SG / VW); e += blockDim.x) {
        int b2 = e / (G::SG / VW), q = e % (G::SG / VW);
        if (!s_act[b2]) continue;
        reinterpret_cast<V*>(tmp + m.offg[s_slot[b2]])[q] = reinterpret_cast<const V*>(sm + b2 * G::SG)[q];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// correct_children (src/m_aX_mg.f90:368-395): per parent, tmp = phi - tmp over
// the whole box, then every child gets phi += prolong2(tmp)
// (mg$D_box_corr_lpl :708-715, a$D_prolong2 with add, src/m_aX_prolong.f90:
// 243-348). One thread per parent interior cell; that cell feeds the 2^D fine
// cells of the child whose quadrant contains it. SUB = the children are on a
// level <= 1 (one child, twice the cells per direction, no offset).
// ---------------------------------------------------------------------------
template <int D, int NC, bool SUB, class T>
__global__ void __launch_bounds__(kThreads)
k_correct(Meta m, BoxSet bs, T* __restrict__ phi, T* __restrict__ tmp, int pull, int homog) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;  // parent geometry
  constexpr int CNC = SUB ? 2 * NC : NC;
  using GC = Geo<D, CNC>;
  constexpr int PER_BOX = G::SI < kThreads ? G::SI : kThreads;
  constexpr int BPC = boxes_per_cta<G::SG, PER_BOX, T>(1);
  using V = typename Vec<T>::type;
  constexpr int VW = Vec<T>::w;
  __shared__ __align__(16) T sm[BPC * G::SG];
  __shared__ int s_slot[BPC];
  __shared__ int s_act[BPC];
  const int groups = (bs.n + BPC - 1) / BPC;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    int nbox;
    if (pull) {
      // The ghost fill of the parents (a$D_gc_box after their up sweeps),
      // stored as the fill stores it, then tmp = phi - tmp from the staged box.
      nbox = stage_boxes<D, NC, T, BPC>(m, bs, grp, phi, sm, s_slot, s_act);
      pull_all_ghosts<D, NC, T>(m, phi, sm, s_slot, s_act, nbox, homog != 0, phi);
    } else {
      nbox = min(BPC, bs.n - grp * BPC);
      if (threadIdx.x < BPC) {
        int s = threadIdx.x < nbox ? box_at(bs, grp * BPC + threadIdx.x) : -1;
        s_slot[threadIdx.x] = s;
        s_act[threadIdx.x] = (s >= 0) ? m.active[m.tree[s]] : 0;
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < nbox * (G::SG / VW); e += blockDim.x) {
      int b = e / (G::SG / VW), q = e % (G::SG / VW);
      if (!s_act[b]) continue;
      long long o = m.offg[s_slot[b]];
      V p = pull ? reinterpret_cast<const V*>(sm + b * G::SG)[q] : reinterpret_cast<const V*>(phi + o)[q];
      V t = reinterpret_cast<const V*>(tmp + o)[q];
      V r;
      if constexpr (VW == 2) {
        r.x = p.x - t.x;
        r.y = p.y - t.y;
      } else {
        r.x = p.x - t.x;
        r.y = p.y - t.y;
        r.z = p.z - t.z;
        r.w = p.w - t.w;
      }
      reinterpret_cast<V*>(sm + b * G::SG)[q] = r;
      reinterpret_cast<V*>(tmp + o)[q] = r;
    }
    __syncthreads();
    int b = threadIdx.x / PER_BOX, q0 = threadIdx.x % PER_BOX;
    if (b < nbox && s_act[b]) {
      int s = s_slot[b];
      const T* t = sm + b * G::SG;
      constexpr int H = NC / 2;
      const int fc = m.first_child[s];
      for (int q = q0; q < G::SI; q += PER_BOX) {
        int ic = q % NC + 1, jc = (q / NC) % NC + 1, kc = (D == 3) ? q / (NC * NC) + 1 : 0;
        int child, li, lj, lk;
        if (SUB) {
          child = fc;
          li = ic;
          lj = jc;
          lk = kc;
        } else {
          int qx = (ic - 1) / H, qy = (jc - 1) / H, qz = (D == 3) ? (kc - 1) / H : 0;
          child = fc + qx + 2 * qy + 4 * qz;
          li = ic - qx * H;
          lj = jc - qy * H;
          lk = (D == 3) ? kc - qz * H : 0;
        }
        T* c = phi + m.offg[child];
        int i_f = 2 * li - 1, j_f = 2 * lj - 1;
        T f0 = t[G::g(ic, jc, kc)];
        T fx = (T)0.125 * (t[G::g(ic + 1, jc, kc)] - t[G::g(ic - 1, jc, kc)]);
        T fy = (T)0.125 * (t[G::g(ic, jc + 1, kc)] - t[G::g(ic, jc - 1, kc)]);
        T fxx = (T)0.03125 * (t[G::g(ic - 1, jc, kc)] - (T)2 * f0 + t[G::g(ic + 1, jc, kc)]);
        T fyy = (T)0.03125 * (t[G::g(ic, jc - 1, kc)] - (T)2 * f0 + t[G::g(ic, jc + 1, kc)]);
        if constexpr (D == 2) {
          T f2 = fxx + fyy;
          long long o00 = GC::g(i_f, j_f, 0), o10 = GC::g(i_f + 1, j_f, 0);
          long long o01 = GC::g(i_f, j_f + 1, 0), o11 = GC::g(i_f + 1, j_f + 1, 0);
          c[o00] = f0 - fx - fy + f2 + c[o00];
          c[o10] = f0 + fx - fy + f2 + c[o10];
          c[o01] = f0 - fx + fy + f2 + c[o01];
          c[o11] = f0 + fx + fy + f2 + c[o11];
        } else {
          int k_f = 2 * lk - 1;
          T fz = (T)0.125 * (t[G::g(ic, jc, kc + 1)] - t[G::g(ic, jc, kc - 1)]);
          T fzz = (T)0.03125 * (t[G::g(ic, jc, kc - 1)] - (T)2 * f0 + t[G::g(ic, jc, kc + 1)]);
          T f2 = fxx + fyy + fzz;
#pragma unroll
          for (int cz = 0; cz < 2; ++cz)
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
              for (int cx = 0; cx < 2; ++cx) {
                long long o = GC::g(i_f + cx, j_f + cy, k_f + cz);
                // f0 -/+ fx -/+ fy -/+ fz + f2 + old, in this order
                T v = f0;
                v = cx ? v + fx : v - fx;
                v = cy ? v + fy : v - fy;
                v = cz ? v + fz : v - fz;
                c[o] = v + f2 + c[o];
              }
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Reductions. Per-tree maxima are accumulated in kStripes slots per tree (box
// index modulo kStripes) so that the boxes of one tree do not all contend for
// one address; k_stripe_reduce folds them. The bit pattern of a non-negative
// double orders like its value, and a NaN orders above every number.
// ---------------------------------------------------------------------------
constexpr int kStripes = 64;

// max that keeps a NaN once seen (fmax would drop it and hide a diverged solve)
__device__ __forceinline__ double nanmax(double a, double b) { return (b > a || b != b) ? b : a; }
__device__ __forceinline__ float nanmaxf(float a, float b) { return (b > a || b != b) ? b : a; }

__device__ __forceinline__ unsigned long long dbits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}

// Exact float -> double conversion with integer instructions (keeps the
// mixed path's conversions off the FP64 pipe).
__device__ __forceinline__ double f2d_exact(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint64_t s = (uint64_t)(b >> 31) << 63;
  const uint32_t e = (b >> 23) & 0xffu;
  const uint32_t m = b & 0x7fffffu;
  uint64_t out;
  if (e == 0xffu) {
    out = s | (0x7ffull << 52) | ((uint64_t)m << 29);
  } else if (e == 0) {
    if (m == 0) {
      out = s;
    } else {  // subnormal float: normalise
      const int p = 31 - __clz((int)m);  // position of the leading one, 0..22
      const uint64_t mant = ((uint64_t)m << (52 - p)) & 0xfffffffffffffull;
      out = s | ((uint64_t)(p - 149 + 1023) << 52) | mant;
    }
  } else {
    out = s | ((uint64_t)(e - 127 + 1023) << 52) | ((uint64_t)m << 29);
  }
  return __longlong_as_double((long long)out);
}

// double -> float, round to nearest even, with integer instructions.
// Results below the float range flush to signed zero.
__device__ __forceinline__ float d2f_rn(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t s = (uint32_t)(b >> 63) << 31;
  const int E = (int)((b >> 52) & 0x7ff);
  const uint64_t M = b & 0xfffffffffffffull;
  if (E == 0x7ff) return __uint_as_float(s | 0x7f800000u | (M ? 0x400000u : 0u));
  const int e = E - 1023 + 127;
  if (e >= 255) return __uint_as_float(s | 0x7f800000u);
  if (e <= 0) {
    if (E == 0 || e < -24) return __uint_as_float(s);
    // subnormal float result
    const uint64_t full = M | (1ull << 52);
    const int shift = 29 + (1 - e);
    const uint64_t q = full >> shift;
    const uint64_t rem = full & ((1ull << shift) - 1);
    const uint64_t half = 1ull << (shift - 1);
    const uint32_t r = (uint32_t)q + ((rem > half || (rem == half && (q & 1))) ? 1u : 0u);
    return __uint_as_float(s | r);
  }
  const uint32_t m23 = (uint32_t)(M >> 29);
  const uint32_t rem = (uint32_t)(M & ((1u << 29) - 1));
  const uint32_t half = 1u << 28;
  uint32_t out = ((uint32_t)e << 23) | m23;
  out += (rem > half || (rem == half && (m23 & 1))) ? 1u : 0u;
  return __uint_as_float(s | out);
}

// Max over the PER_BOX threads of each box (PER_BOX a power of two), then one
// atomicMax per box into dst (uniform per box, may be null).
template <int PER_BOX, class V>
__device__ __forceinline__ void box_max_atomic(V v, unsigned long long* dst, V* red) {
  constexpr int W = PER_BOX < 32 ? PER_BOX : 32;
  // v >= 0 or NaN: doubles compare by their bit patterns (integer
  // instructions, off the FP64 pipe); floats directly
  auto mx = [](V a, V b) {
    if constexpr (sizeof(V) == 8)
      return dbits(b) > dbits(a) ? b : a;
    else
      return (b > a || b != b) ? b : a;
  };
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) v = mx(v, __shfl_xor_sync(0xffffffffu, v, o));
  auto commit = [&](V x) {
    double dv;
    if constexpr (sizeof(V) == 4)
      dv = f2d_exact(x);
    else
      dv = x;
    atomicMax(dst, dbits(dv));
  };
  if constexpr (PER_BOX <= 32) {
    if ((threadIdx.x & (W - 1)) == 0 && dst) commit(v);
  } else {
    constexpr int WPB = PER_BOX / 32;
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red[warp] = v;
    __syncthreads();
    if ((threadIdx.x % PER_BOX) == 0 && dst) {
      V mm = red[warp];
#pragma unroll
      for (int w = 1; w < WPB; ++w) mm = mx(mm, red[warp + w]);
      commit(mm);
    }
    __syncthreads();
  }
}

static __global__ void k_stripe_reduce(int n_trees, const unsigned long long* __restrict__ norm,
                                unsigned long long* __restrict__ out) {
  pdl_wait();
  pdl_trigger();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_trees) {
    unsigned long long mx = 0;
    for (int k = 0; k < kStripes; ++k) {
      unsigned long long v = norm[(size_t)t * kStripes + k];
      mx = v > mx ? v : mx;
    }
    out[t] = mx;
  }
}

// ---------------------------------------------------------------------------
// Residual tmp = rhs - L(phi) on every box of a set (residual_box,
// src/m_aX_mg.f90:545-559), and optionally max |tmp| over the leaf boxes per
// tree (a$D_tree_max_cc / a$D_tree_min_cc, src/m_aX_utils.f90:468-571).
// ---------------------------------------------------------------------------
template <int D, int NC, class T>
__global__ void __launch_bounds__(kThreads)
k_residual(Meta m, BoxSet bs, const T* __restrict__ phi, const T* __restrict__ rhs,
           T* __restrict__ tmp, unsigned long long* __restrict__ norm_per_tree, int store) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int PER_BOX = G::SI < kThreads ? G::SI : kThreads;
  constexpr int BPC = kThreads / PER_BOX;
  __shared__ double red[kThreads / 32];
  const int groups = (bs.n + BPC - 1) / BPC;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    int b = threadIdx.x / PER_BOX, q0 = threadIdx.x % PER_BOX;
    int bi = grp * BPC + b;
    // max |r| kept as the bit pattern of |r|: a non-negative double orders
    // like its bits (a NaN above every number), so the maximum takes integer
    // instructions instead of FP64 compares on GB300's slow FP64 pipe
    unsigned long long mbits = 0;
    int tr = -1;
    bool leaf = false;
    if (bi < bs.n) {
      int s = box_at(bs, bi);
      const SlotDesc& d = m.desc[s];
      tr = d.tree;
      if (m.active[tr]) {
        leaf = m.first_child[s] < 0;
        const T* bx = phi + d.offg;
        const T inv = Sc<T>::inv(d);
        for (int q = q0; q < G::SI; q += PER_BOX) {
          int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
          T r = rhs[d.offi + q] - lpl_at<D, NC, T>(bx, i, j, k, inv);
          if (store) tmp[d.offg + G::g(i, j, k)] = r;
          const unsigned long long rb = dbits((double)r) & 0x7fffffffffffffffull;
          mbits = rb > mbits ? rb : mbits;
        }
      } else {
        tr = -1;
      }
    }
    const double mx = __longlong_as_double((long long)mbits);
    if (norm_per_tree) {
      // all threads of a PER_BOX segment belong to the same box
      box_max_atomic<PER_BOX, double>(
          mx, (tr >= 0 && leaf) ? norm_per_tree + (size_t)tr * kStripes + (bi & (kStripes - 1)) : nullptr,
          red);
    }
  }
}

// max |v| over the interiors of a set of boxes (variable in interior layout or
// ghosted layout), per tree.
template <int D, int NC, class T>
__global__ void __launch_bounds__(kThreads)
k_maxabs(Meta m, BoxSet bs, const T* __restrict__ v, int ghosted,
         unsigned long long* __restrict__ norm_per_tree) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int PER_BOX = G::SI < 32 ? G::SI : 32;  // one warp per box
  constexpr int BPC = kThreads / PER_BOX;
  __shared__ double red[kThreads / 32];
  const int groups = (bs.n + BPC - 1) / BPC;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    int b = threadIdx.x / PER_BOX, q0 = threadIdx.x % PER_BOX;
    int bi = grp * BPC + b;
    double mx = 0;
    int tr = -1;
    if (bi < bs.n) {
      int s = box_at(bs, bi);
      tr = m.tree[s];
      if (!m.active[tr]) tr = -1;
      if (tr >= 0) {
        for (int q = q0; q < G::SI; q += PER_BOX) {
          int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
          T x = ghosted ? v[m.offg[s] + G::g(i, j, k)] : v[m.offi[s] + q];
          const double ax = __longlong_as_double((long long)(dbits((double)x) & 0x7fffffffffffffffull));
          mx = dbits(ax) > dbits(mx) ? ax : mx;  // |x| >= 0 or NaN: compare the bits
        }
      }
    }
    box_max_atomic<PER_BOX, double>(
        mx, tr >= 0 ? norm_per_tree + (size_t)tr * kStripes + (bi & (kStripes - 1)) : nullptr, red);
  }
}

// Elementwise operations over whole boxes (ghosts included), as the
// reference's full-array utilities do: a$D_box_clear_cc, a$D_box_copy_cc
// (src/m_aX_utils.f90:262-270, :331-339).
template <int D, int NC, class T>
__global__ void __launch_bounds__(kThreads)
k_box_op(Meta m, BoxSet bs, T* __restrict__ dst, const T* __restrict__ src, int op) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  using V = typename Vec<T>::type;
  constexpr int VW = Vec<T>::w;
  constexpr int NV = G::SG / VW;
  const long long total = (long long)bs.n * NV;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int bi = (int)(e / NV), q = (int)(e % NV);
    int s = box_at(bs, bi);
    if (!m.active[m.tree[s]]) continue;
    V* d = reinterpret_cast<V*>(dst + m.offg[s]) + q;
    if (op == 0) {
      V z;
      if constexpr (VW == 2) {
        z.x = 0; z.y = 0;
      } else {
        z.x = 0; z.y = 0; z.z = 0; z.w = 0;
      }
      *d = z;
    } else {
      *d = reinterpret_cast<const V*>(src + m.offg[s])[q];
    }
  }
}

// Restriction of an interior-layout variable (rhs) to the parent, the
// init_phi_rhs step of src/m_aX_mg.f90:530-541 (a$D_restrict_box).
template <int D, int NC, bool SUB, class T>
__global__ void __launch_bounds__(kThreads)
k_restrict_interior(Meta m, BoxSet bs, T* __restrict__ v) {
  pdl_wait();
  pdl_trigger();
  constexpr int H = NC / 2;
  constexpr int PNC = SUB ? NC / 2 : NC;
  constexpr int PER_BOX = D == 2 ? H * H : H * H * H;
  using G = Geo<D, NC>;
  using GP = Geo<D, PNC>;
  const long long total = (long long)bs.n * PER_BOX;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int bi = (int)(e / PER_BOX), q = (int)(e % PER_BOX);
    int s = box_at(bs, bi);
    const SlotDesc& d = m.desc[s];
    if (!m.active[d.tree]) continue;
    int ic = q % H + 1, jc = (q / H) % H + 1, kc = (D == 3) ? q / (H * H) + 1 : 1;
    int off[3] = {0, 0, 0};
    if (!SUB) {
      const int qd = d.qd;
      off[0] = (qd & 1) * H;
      off[1] = ((qd >> 1) & 1) * H;
      off[2] = ((qd >> 2) & 1) * H;
    }
    const T* f = v + d.offi;
    T acc = 0;
    constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
    for (int kk = 0; kk < KK; ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii) acc = acc + f[G::in(2 * ic - 1 + ii, 2 * jc - 1 + jj, 2 * kc - 1 + kk)];
    const T w = (D == 2) ? (T)0.25 : (T)0.125;
    v[m.offi[d.parent] + GP::in(off[0] + ic, off[1] + jc, off[2] + kc)] = w * acc;
  }
}

// ---------------------------------------------------------------------------
// Fixed-point Laplacian for the defect. GB300 issues few FP64 instructions
// per clock, and the defect's FP64 sum of 2D + 1 cells per cell kept that
// pipe 80 % busy. Instead, every cell the stencil reads (interior and face
// ghosts) of a box is scaled to a 64-bit integer X = v * 2^(1081 - emax),
// emax the largest biased exponent among them: |X| < 2^59, the neighbour sum
// minus 2D X_c is exact in 64-bit integers (|S| < 12 * 2^59), and S times
// 2^(emax - 1081) is made a double by integer operations (truncated to 53
// bits). The only rounding is the truncation of cells far below the box's
// largest (below 2^-59 of it) and that final truncation; the FP64 sum rounds
// every partial sum to 53 bits relative to |u|, so this is the more accurate
// of the two. One FP64 fused multiply-add per cell remains: r = f - S/dx^2.
// Every finite box can be scaled so (from_fx's exponent emax + 5 - lz stays
// in [emax - 58, emax + 4]); a box holding an infinity or NaN takes the FP64
// sum, which carries it into the residual.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int dexp(double v) {
  return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ff);
}
// v * 2^(1081 - emax), truncated toward zero (E(v) <= emax).
__device__ __forceinline__ long long to_fx(double v, int emax) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((b >> 52) & 0x7ff);
  if (E == 0) return 0;  // zero or subnormal (below 2^-1022)
  const unsigned long long M6 = ((b & 0xfffffffffffffull) | (1ull << 52)) << 6;  // < 2^59
  const int dsh = emax - E;  // >= 0
  const unsigned long long X = dsh < 64 ? (M6 >> dsh) : 0ull;
  return (b >> 63) ? -(long long)X : (long long)X;
}
// S * 2^(emax - 1081) as a double (|S| < 2^63; mantissa truncated).
__device__ __forceinline__ double from_fx(long long S, int emax) {
  if (S == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)S & (1ull << 63);
  unsigned long long T = S < 0 ? 0ull - (unsigned long long)S : (unsigned long long)S;
  const int lz = __clzll((long long)T);
  T <<= lz;  // leading one at bit 63
  const unsigned long long mant = (T >> 11) & 0xfffffffffffffull;
  const unsigned long long bexp = (unsigned long long)(emax + 5 - lz);
  return __longlong_as_double((long long)(sgn | (bexp << 52) | mant));
}
// Whether ghosted position e of a box is read by the 2D+1-point stencil
// (interior or face ghost; edge and corner ghosts are never filled).
template <int D, int NC>
__device__ __forceinline__ bool stencil_reads(int e) {
  using G = Geo<D, NC>;
  const int i = e % G::NG, j = (e / G::NG) % G::NG, k = (D == 3) ? e / (G::NG * G::NG) : 1;
  const int out = (i == 0 || i == NC + 1) + (j == 0 || j == NC + 1) + (k == 0 || k == NC + 1);
  return out <= 1;
}

// ---------------------------------------------------------------------------
// Mixed precision: FP64 defect correction around FP32 V-cycles.
//
// k_defect: on every leaf, r = f - L(u) with an FP64 sum and fused
// multiply-adds, stored as the FP32 right-hand side of the correction cycle,
// and max |r| per tree (k_defect_warp below is the default form, with the
// fixed-point Laplacian). The ghost cells of u are recomputed here from the
// current state: neighbours' cells,
// physical boundaries, and at refinement boundaries the coarse neighbour's
// cell that the parent's ghost cell would hold (two hops: the parent's
// neighbour exists by 2:1 balance and is a leaf).
// ---------------------------------------------------------------------------
template <int D, int NC>
__global__ void __launch_bounds__(kThreads)
k_defect(Meta m, BoxSet bs, const double* __restrict__ u, const double* __restrict__ f,
         float* __restrict__ r32, unsigned long long* __restrict__ norm_per_tree) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int PER_BOX = G::SI < kThreads ? G::SI : kThreads;
  constexpr int BPC = boxes_per_cta<G::SG, PER_BOX, double>(1);
  __shared__ __align__(16) double sm[BPC * G::SG];
  __shared__ int s_slot[BPC];
  __shared__ int s_act[BPC];
  __shared__ float red[kThreads / 32];
  const int groups = (bs.n + BPC - 1) / BPC;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    const int nbox = stage_boxes<D, NC, double, BPC>(m, bs, grp, u, sm, s_slot, s_act);
    for (int e = threadIdx.x; e < nbox * G::NNB * G::NF; e += blockDim.x) {
      const int b = e / (G::NNB * G::NF);
      const int r = e % (G::NNB * G::NF);
      const int fc = r / G::NF, lin = r % G::NF;
      const int a = lin % NC + 1, c = lin / NC + 1;
      if (!s_act[b]) continue;
      const int s = s_slot[b];
      const SlotDesc& d = m.desc[s];
      const double* bx = sm + b * G::SG;
      auto own = [&](int i, int j, int k) { return bx[G::g(i, j, k)]; };
      const Face<D, NC> F(fc, a, c);
      const int code = d.code[fc];
      double v;
      if (code >= 0) {
        v = u[d.nbo[fc] + G::g(F.ni, F.nj, F.nk)];
      } else if (code == kFaceRefinement) {
        const double g0 = u[m.nbo2[s * G::NNB + fc] + parent_cell<D, NC>(F, fc, d.qd, true)];
        v = rb_value<D, NC, double>(F, fc, g0, own);
      } else {
        double bv = 0;
        if (d.nbo[fc] >= 0) bv = m.bcval[d.nbo[fc] + ((D == 2) ? (a - 1) : (a - 1) + NC * (c - 1))];
        v = bc_value<double>(code, fc, bv, own(F.ai, F.aj, F.ak), d.dr);
      }
      sm[b * G::SG + G::g(F.gi, F.gj, F.gk)] = v;
    }
    __syncthreads();
    const int b = threadIdx.x / PER_BOX, q0 = threadIdx.x % PER_BOX;
    float mx = 0.f;
    int tr = -1;
    if (b < nbox && s_act[b]) {
      const SlotDesc& d = m.desc[s_slot[b]];
      tr = d.tree;
      const double* bx = sm + b * G::SG;
      const double ninv = -d.inv_dx2;
      for (int q = q0; q < G::SI; q += PER_BOX) {
        const int i = q % NC + 1, j = (q / NC) % NC + 1, k = (D == 3) ? q / (NC * NC) + 1 : 0;
        double sum;
        if constexpr (D == 2)
          sum = ((bx[G::g(i - 1, j, 0)] + bx[G::g(i + 1, j, 0)]) + bx[G::g(i, j - 1, 0)]) + bx[G::g(i, j + 1, 0)];
        else
          sum = ((((bx[G::g(i - 1, j, k)] + bx[G::g(i + 1, j, k)]) + bx[G::g(i, j - 1, k)]) +
                  bx[G::g(i, j + 1, k)]) + bx[G::g(i, j, k - 1)]) + bx[G::g(i, j, k + 1)];
        const double t = fma(-(double)(2 * D), bx[G::g(i, j, k)], sum);
        const double rr = fma(ninv, t, f[d.offi + q]);
        const float r = d2f_rn(rr);
        r32[d.offi + q] = r;
        mx = nanmaxf(mx, fabsf(r));
      }
    }
    box_max_atomic<PER_BOX, float>(
        mx,
        (tr >= 0) ? norm_per_tree + (size_t)tr * kStripes + ((grp * BPC + b) & (kStripes - 1)) : nullptr,
        red);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// k_defect_fx: k_defect with the fixed-point Laplacian. A 256-thread block
// takes LPB leaves per iteration (one group of LT = SI / CR threads per leaf,
// at most 256: CR cells per thread, more in boxes of over 256 CR cells) in a
// three-deep software
// pipeline, so that every load of an iteration's leaves is in flight while
// the block computes the iteration before: at iteration k the block waits for
// the copies issued at k - 1 (the leaves' u, interior rows only, and the next
// leaves' descriptors), issues iteration k + 1's u and k + 2's descriptors
// (cp.async), loads k + 1's ghost sources and f into registers, and computes
// iteration k: ghost cells from the sources and each leaf's own cells, each
// leaf's largest exponent of the cells the stencil reads, those cells in
// fixed point in place, then r = f - S/dx^2 for its cells. A leaf holding an
// infinity or NaN takes the FP64 sum instead. Boxes of at least 32 cells
// (smaller ones use k_defect).
// ---------------------------------------------------------------------------
template <int D, int NC, int CR>
struct DefectFxCfg {
  using G = Geo<D, NC>;
  static constexpr int LT = G::SI / CR < 256 ? G::SI / CR : 256;  // threads of a leaf
  static constexpr int LPB = 256 / LT;                  // leaves of an iteration
  static constexpr int T = LT * LPB;                    // threads of a block
  static constexpr int SEG = LT < 32 ? LT : 32;         // lanes of a reduction segment (one leaf's, or a warp)
  static constexpr int SPL = LT / SEG;                  // segments of a leaf
  static constexpr int NSEG = T / SEG;                  // segments of a block
  static constexpr int CPT = G::SI / LT;                // interior cells per thread
  static constexpr int NEED = 2 * D * G::NF;            // face ghosts of a leaf
  static constexpr int IPT = (NEED + LT - 1) / LT;      // face ghosts per thread
  static constexpr int SPT = (G::SG + LT - 1) / LT;     // ghosted cells per thread
  static constexpr int NPL = D == 3 ? NC : 1;           // interior planes of a box
  static constexpr int PCH = NC * G::NG * 8 / 16;       // 16-byte chunks of a plane's interior rows
  // static shared memory: two staged leaves per iteration slot, three
  // descriptor slots, the segments' exponents and maxima (at most 48 KB)
  static constexpr int SMEM = 2 * LPB * G::SG * 8 + 3 * LPB * (int)sizeof(SlotDesc) + 2 * NSEG * 8;
  static constexpr bool OK = LT >= 16 && (LT % 32 == 0 || 32 % LT == 0) && 256 % LT == 0 &&
                             G::SI % LT == 0 && (G::NG * 8) % 16 == 0 && SPT <= 32 && SMEM <= 48 * 1024;
};

template <int D, int NC, int CR>
__global__ void __launch_bounds__(256, CR >= 4 ? 4 : 5)
k_defect_fx(Meta m, BoxSet bs, const double* __restrict__ u, const double* __restrict__ f,
            float* __restrict__ r32, unsigned long long* __restrict__ norm_per_tree) {
  pdl_trigger();  // the first descriptors are copied before pdl_wait() (they never change)
  using C = DefectFxCfg<D, NC, CR>;
  using G = Geo<D, NC>;
  static_assert(C::OK, "k_defect_fx block shape");
  constexpr int L = C::LPB;
  __shared__ __align__(16) double sb[2][L][G::SG];
  __shared__ __align__(16) SlotDesc sd[3][L];
  __shared__ int s_em[2][C::NSEG];
  __shared__ float s_mx[2][C::NSEG];
  const int tid = threadIdx.x;
  const int seg = tid / C::SEG, first_of_seg = (tid % C::SEG) == 0;
  const int lb = tid / C::LT, lt = tid % C::LT;  // this thread's leaf in an iteration, its thread there
  const int groups = (bs.n + L - 1) / L;
  const int first = blockIdx.x, step = gridDim.x;
  const int my = first < groups ? (groups - 1 - first) / step + 1 : 0;
  if (my == 0) {
    pdl_wait();
    return;
  }
  unsigned rmask = 0;  // ghosted cells lt + LT j that the stencil reads
#pragma unroll
  for (int j = 0; j < C::SPT; ++j) {
    const int e = lt + C::LT * j;
    if (e < G::SG && stencil_reads<D, NC>(e)) rmask |= 1u << j;
  }
  // index in the set of this thread's leaf at iteration k, and its slot
  // (-1 past the end of the set)
  auto leaf_of = [&](int k) { return (first + k * step) * L + lb; };
  auto slot_of = [&](int k) {
    const int li = leaf_of(k);
    return li < bs.n ? box_at(bs, li) : -1;
  };
  auto copy_desc = [&](int k, int s) {
    if (s >= 0 && lt < (int)sizeof(SlotDesc) / 16)
      cp_async16(reinterpret_cast<char*>(&sd[k % 3][lb]) + 16 * lt,
                 reinterpret_cast<const char*>(m.desc + s) + 16 * lt);
  };
  // A leaf's rows j = 1..NC of the planes k = 1..NC (the one plane in 2-D):
  // its interior with the x ghosts between the rows, contiguous per plane.
  // The ghost planes and rows are not read: every face ghost the stencil
  // reads is computed from its sources below, edges and corners are unused.
  auto copy_box = [&](int k, int s) {
    if (s < 0) return;
    const char* src = reinterpret_cast<const char*>(u + sd[k % 3][lb].offg);
    char* dst = reinterpret_cast<char*>(sb[k & 1][lb]);
    for (int c = lt; c < C::NPL * C::PCH; c += C::LT) {
      const int off = 8 * (G::NG + (D == 3 ? (c / C::PCH + 1) * G::NG * G::NG : 0)) + 16 * (c % C::PCH);
      cp_async16(dst + off, src + off);
    }
  };
  // This thread's face ghosts (fixed for every leaf): face (-1: none), ghost,
  // neighbour's and adjacent cell positions, index in the face; and its cells.
  int it_f[C::IPT], it_g[C::IPT], it_n[C::IPT], it_a[C::IPT], it_lin[C::IPT];
#pragma unroll
  for (int j = 0; j < C::IPT; ++j) {
    const int r = lt + C::LT * j;
    const int rr = r < C::NEED ? r : 0;
    const int fc = rr / G::NF, lin = rr % G::NF;
    const Face<D, NC> F(fc, lin % NC + 1, lin / NC + 1);
    it_f[j] = r < C::NEED ? fc : -1;
    it_g[j] = G::g(F.gi, F.gj, F.gk);
    it_n[j] = G::g(F.ni, F.nj, F.nk);
    it_a[j] = G::g(F.ai, F.aj, F.ak);
    it_lin[j] = lin;
  }
  int cpos[C::CPT];
#pragma unroll
  for (int c = 0; c < C::CPT; ++c) {
    const int q = lt + C::LT * c;
    cpos[c] = G::g(q % NC + 1, (q / NC) % NC + 1, (D == 3) ? q / (NC * NC) + 1 : 0);
  }
  // Ghost sources and f of this thread's leaf at iteration k (its
  // descriptor has landed), slot s (-1: none).
  auto fetch = [&](int k, int s, double (&gv)[C::IPT], double (&fv)[C::CPT]) {
#pragma unroll
    for (int j = 0; j < C::IPT; ++j) gv[j] = 0.0;
#pragma unroll
    for (int c = 0; c < C::CPT; ++c) fv[c] = 0.0;
    if (s < 0) return;
    const SlotDesc& d = sd[k % 3][lb];
#pragma unroll
    for (int j = 0; j < C::IPT; ++j) {
      const int fc = it_f[j];
      if (fc < 0) continue;
      const int code = d.code[fc];
      if (code >= 0) {
        gv[j] = u[d.nbo[fc] + it_n[j]];
      } else if (code == kFaceRefinement) {
        const Face<D, NC> F(fc, it_lin[j] % NC + 1, it_lin[j] / NC + 1);
        gv[j] = u[m.nbo2[(size_t)s * G::NNB + fc] + parent_cell<D, NC>(F, fc, d.qd, true)];
      } else if (d.nbo[fc] >= 0) {
        gv[j] = m.bcval[d.nbo[fc] + it_lin[j]];
      }
    }
#pragma unroll
    for (int c = 0; c < C::CPT; ++c) fv[c] = f[d.offi + lt + C::LT * c];
  };
  // max |r| of this thread's leaf at iteration k (per-segment maxima in
  // s_mx[k & 1]) into the stripe of its tree (tree < 0: inactive, nothing to
  // add); the leaf's first thread only
  auto commit_norm = [&](int k, int tree) {
    if (lt == 0 && tree >= 0) {
      float mx = 0.f;
#pragma unroll
      for (int w = 0; w < C::SPL; ++w) mx = nanmaxf(mx, s_mx[k & 1][lb * C::SPL + w]);
      atomicMax(norm_per_tree + (size_t)tree * kStripes + (leaf_of(k) & (kStripes - 1)), dbits(f2d_exact(mx)));
    }
  };

  // prologue: descriptors of iteration 0, then its u and the descriptors of iteration 1
  int s_cur = slot_of(0);
  copy_desc(0, s_cur);
  int s_next = my > 1 ? slot_of(1) : -1;
  if (my > 1) copy_desc(1, s_next);
  cp_async_commit();
  int s_after = my > 2 ? slot_of(2) : -1;
  cp_async_wait<0>();
  __syncthreads();
  pdl_wait();  // u and the flags may have been written by the previous kernel
  copy_box(0, s_cur);
  cp_async_commit();
  double gc[C::IPT], gn[C::IPT], fcv[C::CPT], fnv[C::CPT];
  fetch(0, s_cur, gc, fcv);
  int tree_prev = -1;  // tree of this thread's previous leaf if it was active (a leaf's first thread)

  for (int k = 0; k < my; ++k) {
    cp_async_wait<0>();
    __syncthreads();  // iteration k's u and k + 1's descriptors have landed; iteration k - 1 is done
    if (k > 0) commit_norm(k - 1, tree_prev);
    if (k + 1 < my) copy_box(k + 1, s_next);
    if (k + 2 < my) copy_desc(k + 2, s_after);
    cp_async_commit();
    const int s_far = k + 3 < my ? slot_of(k + 3) : -1;
    if (k + 1 < my) fetch(k + 1, s_next, gn, fnv);
    const SlotDesc& d = sd[k % 3][lb];
    double* bx = sb[k & 1][lb];
    // uniform over a leaf's threads (whole warps, or a segment of a warp)
    const bool act = s_cur >= 0 && m.active[d.tree] != 0;
    tree_prev = act ? d.tree : -1;
    if (act) {
#pragma unroll
      for (int j = 0; j < C::IPT; ++j) {
        const int fc = it_f[j];
        if (fc < 0) continue;
        const int code = d.code[fc];
        double v = gc[j];
        if (code == kFaceRefinement) {
          const Face<D, NC> F(fc, it_lin[j] % NC + 1, it_lin[j] / NC + 1);
          auto own = [&](int i, int jj, int kk) { return bx[G::g(i, jj, kk)]; };
          v = rb_value<D, NC, double>(F, fc, gc[j], own);
        } else if (code < 0) {
          v = bc_value<double>(code, fc, gc[j], bx[it_a[j]], d.dr);
        }
        bx[it_g[j]] = v;
      }
    }
    __syncthreads();
    {
      // every lane reduces (0 for an inactive leaf): a segment may be half
      // a warp whose other half is another leaf
      int em = 0;
      if (act) {
#pragma unroll
        for (int j = 0; j < C::SPT; ++j)
          if (rmask & (1u << j)) em = max(em, dexp(bx[lt + C::LT * j]));
      }
      if constexpr (C::SEG == 32) {
        em = __reduce_max_sync(0xffffffffu, em);
      } else {
#pragma unroll
        for (int o = C::SEG / 2; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
      }
      if (act && first_of_seg) s_em[k & 1][seg] = em;
    }
    __syncthreads();
    int emax = 0;
    if (act) {
#pragma unroll
      for (int w = 0; w < C::SPL; ++w) emax = max(emax, s_em[k & 1][lb * C::SPL + w]);
    }
    // the leaf's cells in fixed point in place (a leaf with an infinity or
    // NaN keeps its doubles); every thread reaches the barrier
    const bool fx = act && emax != 0x7ff;
    long long* X = reinterpret_cast<long long*>(bx);
    if (fx) {
#pragma unroll
      for (int j = 0; j < C::SPT; ++j)
        if (rmask & (1u << j)) X[lt + C::LT * j] = to_fx(bx[lt + C::LT * j], emax);
    }
    __syncthreads();
    float mx = 0.f;
    if (act) {
      const double ninv = -d.inv_dx2;
      float* rb = r32 + d.offi;
      if (fx) {
#pragma unroll
        for (int c = 0; c < C::CPT; ++c) {
          const int q = lt + C::LT * c;
          const long long* x = X + cpos[c];
          constexpr int OY = G::NG, OZ = G::NG * G::NG;
          const long long xc = x[0];
          long long Sx;
          if constexpr (D == 2)
            Sx = x[-1] + x[1] + x[-OY] + x[OY] - 4 * xc;
          else
            Sx = x[-1] + x[1] + x[-OY] + x[OY] + x[-OZ] + x[OZ] - 6 * xc;
          const float r = __double2float_rn(fma(ninv, from_fx(Sx, emax), fcv[c]));
          rb[q] = r;
          mx = nanmaxf(mx, fabsf(r));
        }
      } else {
#pragma unroll
        for (int c = 0; c < C::CPT; ++c) {
          const int q = lt + C::LT * c;
          const int i = q % NC + 1, j = (q / NC) % NC + 1, kz = (D == 3) ? q / (NC * NC) + 1 : 0;
          double sum;
          if constexpr (D == 2)
            sum = ((bx[G::g(i - 1, j, 0)] + bx[G::g(i + 1, j, 0)]) + bx[G::g(i, j - 1, 0)]) + bx[G::g(i, j + 1, 0)];
          else
            sum = ((((bx[G::g(i - 1, j, kz)] + bx[G::g(i + 1, j, kz)]) + bx[G::g(i, j - 1, kz)]) +
                    bx[G::g(i, j + 1, kz)]) + bx[G::g(i, j, kz - 1)]) + bx[G::g(i, j, kz + 1)];
          const double t = fma(-(double)(2 * D), bx[G::g(i, j, kz)], sum);
          const float r = __double2float_rn(fma(ninv, t, fcv[c]));
          rb[q] = r;
          mx = nanmaxf(mx, fabsf(r));
        }
      }
    }
    // every lane reduces within its segment (0 for an inactive leaf)
#pragma unroll
    for (int o = C::SEG / 2; o > 0; o >>= 1) mx = nanmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (act && first_of_seg) s_mx[k & 1][seg] = mx;
#pragma unroll
    for (int j = 0; j < C::IPT; ++j) gc[j] = gn[j];
#pragma unroll
    for (int c = 0; c < C::CPT; ++c) fcv[c] = fnv[c];
    s_cur = s_next;
    s_next = s_after;
    s_after = s_far;
  }
  __syncthreads();
  commit_norm(my - 1, tree_prev);
}

// u += e over the interiors of the leaves (FP64 accumulate of the FP32
// correction). One thread per row of NC cells: the slot lookups are made once
// per row. The whole ghosted row (NC + 2 cells, an even count from an even
// offset: 16-byte aligned doubles, 8-byte aligned floats) moves in vector
// loads and stores, with its two ghost cells written back unchanged; the
// sectors touched are those of the interior row alone.
template <int D, int NC>
__global__ void __launch_bounds__(kThreads)
k_accumulate(Meta m, BoxSet bs, double* __restrict__ u, const float* __restrict__ e) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  static_assert(G::NG % 2 == 0, "rows of an even number of cells");
  constexpr int ROWS = G::SI / NC;  // rows of a box
  constexpr int H = G::NG / 2;      // vector pairs of a ghosted row
  const long long total = (long long)bs.n * ROWS;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int bi = (int)(x / ROWS), row = (int)(x % ROWS);
    const int s = box_at(bs, bi);
    if (!m.active[m.tree[s]]) continue;
    const int j = row % NC + 1, k = (D == 3) ? row / NC + 1 : 0;
    const long long o = m.offg[s] + G::g(0, j, k);
    double2* ur = reinterpret_cast<double2*>(u + o);
    const float2* er = reinterpret_cast<const float2*>(e + o);
    double2 uv[H];
    float2 ev[H];
#pragma unroll
    for (int i = 0; i < H; ++i) {
      uv[i] = ur[i];
      ev[i] = er[i];
    }
    // cell 0 and cell NG - 1 are ghosts
#pragma unroll
    for (int i = 0; i < H; ++i) {
      if (i > 0) uv[i].x = uv[i].x + f2d_exact(ev[i].x);
      if (i < H - 1) uv[i].y = uv[i].y + f2d_exact(ev[i].y);
    }
#pragma unroll
    for (int i = 0; i < H; ++i) ur[i] = uv[i];
  }
}

// Parents of a level >= 1: the increment of a parent cell is the restriction
// (2^D-cell average) of its children's increments -- the correction e on leaf
// children, the increment stored here by the previous call on parent children.
// The parent's u gets the increment in FP64 and the increment replaces e on the
// parent, so that after the finest-to-coarsest pass every parent holds the
// restriction of its children, as at the fixed point of the FAS cycle.
template <int D, int NC>
__global__ void __launch_bounds__(kThreads)
k_restrict_increment(Meta m, BoxSet bs, double* __restrict__ u, float* __restrict__ e) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int H = NC / 2;
  const long long total = (long long)bs.n * G::SI;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int bi = (int)(x / G::SI), q = (int)(x % G::SI);
    const int s = box_at(bs, bi);
    if (!m.active[m.tree[s]]) continue;
    const int ic = q % NC + 1, jc = (q / NC) % NC + 1, kc = (D == 3) ? q / (NC * NC) + 1 : 0;
    const int qx = (ic - 1) / H, qy = (jc - 1) / H, qz = (D == 3) ? (kc - 1) / H : 0;
    const int child = m.first_child[s] + qx + 2 * qy + 4 * qz;
    const int li = ic - qx * H, lj = jc - qy * H, lk = (D == 3) ? kc - qz * H : 0;
    const float* ce = e + m.offg[child];
    float acc = 0.f;
    constexpr int KK = (D == 3) ? 2 : 1;
#pragma unroll
    for (int kk = 0; kk < KK; ++kk)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
          acc += ce[G::g(2 * li - 1 + ii, 2 * lj - 1 + jj, (D == 3) ? 2 * lk - 1 + kk : 0)];
    const float inc = acc * ((D == 2) ? 0.25f : 0.125f);
    const long long o = m.offg[s] + G::g(ic, jc, kc);
    e[o] = inc;
    u[o] = u[o] + f2d_exact(inc);
  }
}

// Right-hand side from a sum of Gaussians a*exp(-|r-c|^2/s^2), or their
// Laplacian (lpl), at the cell centres of a slot range of one tree
// (the source of examples/m_gaussians.f90:64-102), evaluated on the device.
// A Gaussian factors over the axes, exp(-|x|^2) = exp(-x^2) exp(-y^2)
// exp(-z^2), and a box's cell centres lie on NC coordinates per axis: one
// block per box evaluates the factors and squares along each axis (D * NC
// exponentials and divisions per Gaussian instead of NC^D), combines those
// of y and z over the transverse positions, and each cell takes one sum and
// one product of them. GB300 runs FP64 exponentials and divisions slowly; this way the
// source of a 256^3 tree takes a fraction of the time. The factored form
// differs from exp of the sum by a few roundings (relative 1e-15).
constexpr int kMaxGauss = 16;
struct GaussSet {
  int n, lpl;
  double g[kMaxGauss * 5];  // per Gaussian: a, s, c_1..c_D
};

template <int D, int NC>
__global__ void __launch_bounds__(kThreads)
k_source(Meta m, BoxSet bs, int tree, const double* __restrict__ rmin, GaussSet gs,
         double* __restrict__ rhs) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  constexpr int NT = D == 3 ? NC * NC : NC;  // transverse (y, z) positions of a box
  __shared__ double s_sq[kMaxGauss][3][NC];  // ((r_d - c_d) / s)^2 at the box's NC coordinates
  __shared__ double s_ex[kMaxGauss][3][NC];  // exp(-that)
  __shared__ double s_sqt[kMaxGauss][NT];    // summed over y (and z)
  __shared__ double s_ext[kMaxGauss][NT];    // multiplied over y (and z)
  __shared__ double s_c4[kMaxGauss];         // 4 / s^2 of each Gaussian
  for (int k = threadIdx.x; k < gs.n; k += blockDim.x) s_c4[k] = 4 / (gs.g[k * (2 + D) + 1] * gs.g[k * (2 + D) + 1]);
  for (int bi = blockIdx.x; bi < bs.n; bi += gridDim.x) {
    const int s = bs.lo + bi;
    if (m.tree[s] != tree) continue;  // the same for the whole block
    const double dr = m.desc[s].dr;
    __syncthreads();  // the previous box's factors are no longer read
    for (int e = threadIdx.x; e < gs.n * D * NC; e += blockDim.x) {
      const int k = e / (D * NC), d = (e / NC) % D, i = e % NC + 1;
      const double* p = gs.g + k * (2 + D);
      const double xx = (rmin[(size_t)s * D + d] + (i - 0.5) * dr - p[2 + d]) / p[1];
      s_sq[k][d][i - 1] = xx * xx;
      s_ex[k][d][i - 1] = exp(-(xx * xx));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < gs.n * NT; e += blockDim.x) {
      const int k = e / NT, t = e % NT, j = t % NC;
      if constexpr (D == 3) {
        const int kz = t / NC;
        s_sqt[k][t] = s_sq[k][1][j] + s_sq[k][2][kz];
        s_ext[k][t] = s_ex[k][1][j] * s_ex[k][2][kz];
      } else {
        s_sqt[k][t] = s_sq[k][1][j];
        s_ext[k][t] = s_ex[k][1][j];
      }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < G::SI; q += blockDim.x) {
      const int i = q % NC, t = q / NC;
      double v = 0;
      for (int k = 0; k < gs.n; ++k) {
        const double xr2 = s_sq[k][0][i] + s_sqt[k][t];
        const double ex = s_ex[k][0][i] * s_ext[k][t];
        if (gs.lpl)
          v = v + gs.g[k * (2 + D)] * (s_c4[k] * (xr2 - 0.5 * D) * ex);
        else
          v = v + gs.g[k * (2 + D)] * ex;
      }
      rhs[bs.i0 + (long long)bi * G::SI + q] = v;
    }
  }
}

// Precision conversion over whole boxes (the coarsest level of the mixed
// cycle is smoothed in FP64).
template <class TD, class TS>
__global__ void k_convert(TD* __restrict__ dst, const TS* __restrict__ src, long long n) {
  pdl_wait();
  pdl_trigger();
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x)
    dst[x] = (TD)src[x];
}

// Scatter / gather between the reference's host box layout (boxes in
// level-list order, each (nc+2)^D, or nc^D when packed) and slot storage.
// host_interior: the host buffer holds only interiors. dev_ghosted: the device
// variable has ghost cells (phi, tmp) or not (rhs).
template <int D, int NC, class T>
__global__ void k_scatter(Meta m, const int* __restrict__ slots, int n,
                          const double* __restrict__ src, T* __restrict__ dst, int host_interior,
                          int dev_ghosted) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  const int per = host_interior ? G::SI : G::SG;
  const long long total = (long long)n * per;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    int bi = (int)(x / per), q = (int)(x % per);
    int s = slots[bi];
    int i, j, k;
    if (host_interior) {
      i = q % NC + 1;
      j = (q / NC) % NC + 1;
      k = (D == 3) ? q / (NC * NC) + 1 : 0;
    } else {
      i = q % G::NG;
      j = (q / G::NG) % G::NG;
      k = (D == 3) ? q / (G::NG * G::NG) : 0;
    }
    bool interior = i >= 1 && i <= NC && j >= 1 && j <= NC && (D == 2 || (k >= 1 && k <= NC));
    if (dev_ghosted) {
      dst[m.offg[s] + G::g(i, j, k)] = (T)src[x];
    } else if (interior) {
      dst[m.offi[s] + G::in(i, j, k)] = (T)src[x];
    }
  }
}

template <int D, int NC, class T>
__global__ void k_gather(Meta m, const int* __restrict__ slots, int n, const T* __restrict__ src,
                         double* __restrict__ dst, int host_interior, int dev_ghosted) {
  pdl_wait();
  pdl_trigger();
  using G = Geo<D, NC>;
  const int per = host_interior ? G::SI : G::SG;
  const long long total = (long long)n * per;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    int bi = (int)(x / per), q = (int)(x % per);
    int s = slots[bi];
    int i, j, k;
    if (host_interior) {
      i = q % NC + 1;
      j = (q / NC) % NC + 1;
      k = (D == 3) ? q / (NC * NC) + 1 : 0;
    } else {
      i = q % G::NG;
      j = (q / G::NG) % G::NG;
      k = (D == 3) ? q / (G::NG * G::NG) : 0;
    }
    bool interior = i >= 1 && i <= NC && j >= 1 && j <= NC && (D == 2 || (k >= 1 && k <= NC));
    double v = 0;
    if (dev_ghosted)
      v = (double)src[m.offg[s] + G::g(i, j, k)];
    else if (interior)
      v = (double)src[m.offi[s] + G::in(i, j, k)];
    dst[x] = v;
  }
}

// Keeps the stream busy for about ns nanoseconds (one thread sleeping in a
// loop of at most ns / 1000 + 1000 rounds). The event profiler launches it
// ahead of each solve iteration, so that the host has enqueued the
// iteration's launches before the device reaches them and the events time the
// kernels, not the rate at which the host launches them.
static __global__ void k_hold(long long ns) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (long long r = 0; r < ns / 1000 + 1000; ++r) {
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if ((long long)(t - t0) >= ns) break;
    __nanosleep(1000);
  }
}

// Per-tree convergence bookkeeping on the device: a tree stays active while
// max|r| > tol * max|f|; a non-finite residual stops it and marks it failed.
static __global__ void k_check(int n_trees, const unsigned long long* __restrict__ rnorm,
                        const double* __restrict__ fmax, double tol, int* __restrict__ active,
                        int* __restrict__ failed, int* __restrict__ n_active_out, const int* __restrict__ err,
                        int* __restrict__ cycles, unsigned long long* __restrict__ final_r, int count_cycle) {
  pdl_wait();
  pdl_trigger();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) n_active_out[1] = *err;  // read back with the count
  if (t < n_trees) {
    double r = __longlong_as_double((long long)rnorm[t]);  // reduced over stripes
    int a = active[t];
    if (a) {  // the tree was cycled (unless this is the check before the first cycle)
      final_r[t] = rnorm[t];
      cycles[t] += count_cycle;
    }
    if (a && !(r <= 1.0e300)) {
      a = 0;
      failed[t] = 1;
    } else if (a && r <= tol * fmax[t]) {
      a = 0;
    }
    active[t] = a;
    if (a) atomicAdd(n_active_out, 1);
  }
}

// Sets n ints to v (activity flags).
static __global__ void k_set_int(int* __restrict__ a, int n, int v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

// Loop control of a solve graph (a conditional while node around the
// iterations; one thread each). Words of count: [0] trees still active after
// the last check, [1] the device error word at that check, [2] iterations
// run. k_loop_start enters the loop if a tree is active; k_loop_step, at the
// end of every iteration, repeats it while one is, below max_cycles
// iterations and without a device error.
static __global__ void k_loop_start(cudaGraphConditionalHandle h, int* __restrict__ count, int max_cycles) {
  count[2] = 0;
  cudaGraphSetConditional(h, (count[0] > 0 && max_cycles > 0) ? 1u : 0u);
}
static __global__ void k_loop_step(cudaGraphConditionalHandle h, int* __restrict__ count, int max_cycles) {
  const int c = count[2] + 1;
  count[2] = c;
  cudaGraphSetConditional(h, (count[0] > 0 && c < max_cycles && count[1] == 0) ? 1u : 0u);
}

}  // namespace dev
}  // namespace afv
