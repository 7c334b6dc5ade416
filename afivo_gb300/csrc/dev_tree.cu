// Tree build on the device: a$D_adjust_refinement (src/m_aX_core.f90:452-541)
// with consistent_ref_flags (:628-725), add_children / remove_children
// (:728-787), set_neighbs / find_neighb (:387-422), set_leaves_parents
// (:317-348) and the Morton renumbering of a$D_tidy_up (:238-314,
// src/m_morton.f90), for the built-in refinement criteria. The tree's
// per-id arrays and level lists stay in device memory between passes; only
// the sizes of level lists and the counts that steer the loops come back to
// the host. Every step keeps the host builder's order where it decides ids
// (new ids by an exclusive scan over the level list, renumbering by a sort of
// each level's Morton keys), so ids, links and level lists come out identical
// to host_tree.cpp's.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "afivo_gb300.h"
#include "host_tree.hpp"

namespace afv {
namespace tdev {

enum : int { kRmRef = -1, kKeepRef = 0, kDoRef = 1, kDerefine = -2, kRefine = 2, kNoBox = 0 };

struct Arr {  // per-id arrays, index 0 unused
  int* lvl;
  int* parent;
  int* ncell;
  int* in_use;
  int* ix;         // [id*dim + d]
  int* children;   // [id*nch + c]
  int* nbr;        // [id*nnb + nb]
  double* dr;
  double* rmin;    // [id*dim + d]
};

__device__ __forceinline__ uint64_t spread2(uint32_t v) {
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
__device__ __forceinline__ uint64_t spread3(uint32_t v) {
  uint64_t x = v & 0x1fffffu;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}
__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct Crit {
  int kind, lvl_max, src_lpl, n_gauss, pass;
  double thr, prob;
  unsigned long long seed;
  double gauss[16 * 5];
};

// The built-in ref_subr hooks (host_tree.cpp builtin_ref_fn) for one box,
// evaluated by one warp: flag is read and written like the hook's argument.
__device__ void criterion(const Arr& a, int dim, int id, const Crit& c, int* flag, int lane) {
  const int lvl = a.lvl[id];
  switch (c.kind) {
    case AFV_REF_UNIFORM:
      if (lane == 0 && lvl < c.lvl_max) *flag = kDoRef;
      return;
    case AFV_REF_SOURCE: {
      if (lvl >= c.lvl_max) return;
      const int nc = a.ncell[id];
      const double dr = a.dr[id], dr2 = dr * dr;
      const int n = dim == 3 ? nc * nc * nc : nc * nc;
      bool hit = false;
      for (int q = lane; q < n && !hit; q += 32) {
        const int cix[3] = {q % nc + 1, (q / nc) % nc + 1, q / (nc * nc) + 1};
        double r[3];
        for (int d = 0; d < dim; ++d) r[d] = a.rmin[(size_t)id * dim + d] + (cix[d] - 0.5) * dr;
        double s = 0;
        for (int k = 0; k < c.n_gauss; ++k) {
          const double* p = c.gauss + k * (2 + dim);
          double xr2 = 0;
          for (int d = 0; d < dim; ++d) {
            const double x = (r[d] - p[2 + d]) / p[1];
            xr2 = xr2 + x * x;
          }
          if (c.src_lpl)
            s = s + p[0] * (4 / (p[1] * p[1]) * (xr2 - 0.5 * dim) * exp(-xr2));
          else
            s = s + p[0] * exp(-xr2);
        }
        if (fabs(s) * dr2 > c.thr) hit = true;
      }
      if (__any_sync(0xffffffffu, hit) && lane == 0) *flag = kDoRef;
      return;
    }
    default: {  // AFV_REF_RANDOM, AFV_REF_RANDOM_RM
      if (lane != 0) return;
      uint64_t h = mix(c.seed ^ 0xA5A5A5A5ull);
      h = mix(h ^ (uint64_t)(uint32_t)c.pass);
      h = mix(h ^ (uint64_t)(uint32_t)lvl);
      for (int d = 0; d < dim; ++d) h = mix(h ^ (uint64_t)(uint32_t)a.ix[(size_t)id * dim + d]);
      const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
      if (u < c.prob && lvl < c.lvl_max)
        *flag = kDoRef;
      else if (c.kind == AFV_REF_RANDOM_RM)
        *flag = kRmRef;
      return;
    }
  }
}

__device__ __forceinline__ int ichild_of(const Arr& a, int dim, int nch, int id) {
  int c = nch;
  for (int d = 0; d < dim; ++d) c -= (a.ix[(size_t)id * dim + d] & 1) << d;
  return c;
}

__global__ void k_fill(int* __restrict__ p, long long n, int v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// consistent_ref_flags, the hook calls (core:639-651): every leaf, and the
// parent of every leaf that is its parent's first child. One warp per leaf.
__global__ void k_criterion(Arr a, int dim, int nch, const int* __restrict__ leaves, int n, Crit c,
                            int* __restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const int warps = (int)(gridDim.x * blockDim.x) >> 5;
  for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < n; w += warps) {
    const int id = leaves[w];
    criterion(a, dim, id, c, &flags[id], lane);
    const int p = a.parent[id];
    if (p > kNoBox && ichild_of(a, dim, nch, id) == 1) criterion(a, dim, p, c, &flags[p], lane);
  }
}

// No refinement beyond lvl_limit (core:660-664).
__global__ void k_clamp(const int* __restrict__ ids, int n, int* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (flags[ids[i]] == kDoRef) flags[ids[i]] = kKeepRef;
}

// 2:1 balance on the leaves of one level (core:667-702); levels finest first.
__global__ void k_balance(Arr a, int nnb, const int* __restrict__ leaves, int n, int* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int id = leaves[i];
    if (flags[id] > kKeepRef) {
      flags[id] = kRefine;
      for (int nb = 0; nb < nnb; ++nb)
        if (a.nbr[(size_t)id * nnb + nb] == kNoBox) {
          const int p_nb = a.nbr[(size_t)a.parent[id] * nnb + nb];
          if (p_nb > kNoBox) flags[p_nb] = kRefine;  // always a box in a 2:1 balanced tree
        }
    } else if (flags[id] == kRmRef) {
      for (int nb = 0; nb < nnb; ++nb) {
        const int v = a.nbr[(size_t)id * nnb + nb];
        if (v > kNoBox && (a.children[(size_t)v * (1 << (nnb / 2))] != kNoBox || flags[v] > kKeepRef)) {
          flags[id] = kKeepRef;
          break;
        }
      }
    }
  }
}

// Derefinement of the parents of one level (core:704-722); levels finest first.
__global__ void k_derefine(Arr a, int nch, const int* __restrict__ parents, int n, int* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int id = parents[i];
    bool all_rm = true;
    for (int c = 0; c < nch; ++c)
      if (flags[a.children[(size_t)id * nch + c]] != kRmRef) all_rm = false;
    flags[id] = (all_rm && flags[id] <= kKeepRef) ? kDerefine : kKeepRef;
  }
}

// Counts of kRefine and kDerefine over ids 1..n.
__global__ void k_count(const int* __restrict__ flags, int n, int* __restrict__ out2) {
  int r = 0, d = 0;
  for (int id = 1 + blockIdx.x * blockDim.x + threadIdx.x; id <= n; id += gridDim.x * blockDim.x) {
    r += flags[id] == kRefine;
    d += flags[id] == kDerefine;
  }
  for (int o = 16; o > 0; o >>= 1) {
    r += __shfl_xor_sync(0xffffffffu, r, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out2, r);
    atomicAdd(out2 + 1, d);
  }
}

// Exclusive scan of n ints (values from a predicate of list entries) in one
// block of 1024 threads, each taking a contiguous chunk; total to *sum.
// mode 0: v = (flags[ids[i]] == kRefine && ids[i] <= prev); mode 1: v = has
// children of ids[i].
__global__ void __launch_bounds__(1024) k_scan(Arr a, int nch, const int* __restrict__ ids, int n,
                                               const int* __restrict__ flags, int prev, int mode,
                                               int* __restrict__ out, int* __restrict__ sum) {
  __shared__ int part[1024];
  const int t = threadIdx.x;
  const int chunk = (n + 1023) / 1024;
  const int lo = t * chunk, hi = min(n, lo + chunk);
  auto val = [&](int i) -> int {
    const int id = ids[i];
    return mode == 0 ? (id <= prev && flags[id] == kRefine) : (a.children[(size_t)id * nch] != kNoBox);
  };
  int s = 0;
  for (int i = lo; i < hi; ++i) s += val(i);
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan of the chunk sums
    const int x = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += x;
    __syncthreads();
  }
  int run = t ? part[t - 1] : 0;
  for (int i = lo; i < hi; ++i) {
    out[i] = run;
    run += val(i);
  }
  if (t == 1023) *sum = part[1023];
}

// Position of each id in a level list.
__global__ void k_positions(const int* __restrict__ ids, int n, int* __restrict__ pos) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pos[ids[i]] = i;
}

// add_children (core:752-787) for the refined boxes of a level (new ids from
// their rank in the level list) and remove_children (core:728-749) for the
// derefined ones. The host removes children parent by parent in list order,
// and a removed child whose neighbour is a removed child of another parent
// keeps its link only if its own parent comes first (the later parent finds
// the link already cleared): pos gives the list positions that decide it.
__global__ void k_add_remove(Arr a, int dim, int nch, int nnb, const int* __restrict__ ids, int n,
                             const int* __restrict__ rank, const int* __restrict__ flags, int prev, int hid0,
                             const int* __restrict__ pos) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int id = ids[i];
    if (id > prev) continue;
    if (flags[id] == kRefine) {
      const int c0 = hid0 + 1 + nch * rank[i];
      for (int c = 0; c < nch; ++c) a.children[(size_t)id * nch + c] = c0 + c;
      for (int c = 0; c < nch; ++c) {
        const int k = c0 + c;
        for (int d = 0; d < dim; ++d) {
          const int bit = (c >> d) & 1;
          a.ix[(size_t)k * dim + d] = 2 * a.ix[(size_t)id * dim + d] - 1 + bit;
          a.rmin[(size_t)k * dim + d] = a.rmin[(size_t)id * dim + d] + 0.5 * a.dr[id] * bit * a.ncell[id];
        }
        a.lvl[k] = a.lvl[id] + 1;
        a.parent[k] = id;
        for (int e = 0; e < nch; ++e) a.children[(size_t)k * nch + e] = kNoBox;
        for (int e = 0; e < nnb; ++e) a.nbr[(size_t)k * nnb + e] = kNoBox;
        a.ncell[k] = a.ncell[id];
        a.dr[k] = 0.5 * a.dr[id];
        a.in_use[k] = 1;
      }
      for (int nb = 0; nb < nnb; ++nb) {  // physical boundaries pass to the children on that side
        const int v = a.nbr[(size_t)id * nnb + nb];
        if (v < kNoBox) {
          const int d = nb >> 1, h = nb & 1;
          for (int c = 0; c < nch; ++c)
            if (((c >> d) & 1) == h) a.nbr[(size_t)(c0 + c) * nnb + nb] = v;
        }
      }
    } else if (flags[id] == kDerefine) {
      for (int c = 0; c < nch; ++c) {
        const int k = a.children[(size_t)id * nch + c];
        for (int nb = 0; nb < nnb; ++nb) {
          const int v = a.nbr[(size_t)k * nnb + nb];
          const int rev = (nb & 1) ? nb - 1 : nb + 1;
          if (v <= kNoBox) continue;
          const int pv = a.parent[v];
          if (pv != id && pv <= prev && flags[pv] == kDerefine && pos[pv] < i) continue;
          a.nbr[(size_t)v * nnb + rev] = kNoBox;
        }
        a.in_use[k] = 0;
      }
      for (int c = 0; c < nch; ++c) a.children[(size_t)id * nch + c] = kNoBox;
    }
  }
}

// set_leaves_parents (core:317-348): stable split by has-children.
__global__ void k_split(const int* __restrict__ ids, int n, const int* __restrict__ pos, Arr a, int nch,
                        int* __restrict__ leaves, int* __restrict__ parents) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int id = ids[i];
    if (a.children[(size_t)id * nch] != kNoBox)
      parents[pos[i]] = id;
    else
      leaves[i - pos[i]] = id;
  }
}

// The next level's ids: the children of the parents, in order.
__global__ void k_children_of(Arr a, int nch, const int* __restrict__ parents, int n, int* __restrict__ up) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * nch; i += gridDim.x * blockDim.x)
    up[i] = a.children[(size_t)parents[i / nch] * nch + i % nch];
}

// set_neighbs for the new boxes of a level (core:387-422).
__global__ void k_set_neighbs(Arr a, int dim, int nch, int nnb, const int* __restrict__ ids, int n, int prev) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int id = ids[i];
    if (id <= prev) continue;
    const int c0 = ichild_of(a, dim, nch, id) - 1;
    for (int nb = 0; nb < nnb; ++nb) {
      if (a.nbr[(size_t)id * nnb + nb] != kNoBox) continue;
      const int d = nb >> 1;
      int p = a.parent[id];
      const bool low_child = ((c0 >> d) & 1) == 0, low_nb = (nb & 1) == 0;
      if (low_child == low_nb) p = a.nbr[(size_t)p * nnb + nb];
      // p <= 0 has no children (row 0 of the host arrays holds none)
      const int v = p > kNoBox ? a.children[(size_t)p * nch + (c0 ^ (1 << d))] : kNoBox;
      if (v > kNoBox) {
        a.nbr[(size_t)id * nnb + nb] = v;
        a.nbr[(size_t)v * nnb + ((nb & 1) ? nb - 1 : nb + 1)] = id;
      }
    }
  }
}

// Morton keys of ix - 1 (src/m_morton.f90:33-59) of a level's ids.
__global__ void k_keys(Arr a, int dim, const int* __restrict__ ids, int n, unsigned long long* __restrict__ key,
                       int* __restrict__ val) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int id = ids[i];
    const int* x = a.ix + (size_t)id * dim;
    key[i] = dim == 2 ? (spread2((uint32_t)(x[0] - 1)) | (spread2((uint32_t)(x[1] - 1)) << 1))
                      : (spread3((uint32_t)(x[0] - 1)) | (spread3((uint32_t)(x[1] - 1)) << 1) |
                         (spread3((uint32_t)(x[2] - 1)) << 2));
    val[i] = id;
  }
}

// One merge pass of a stable merge sort (runs of width w into runs of 2w):
// each element's new position is its rank in its own run plus its rank in
// the partner run (lower bound from the left run, upper bound from the right).
__global__ void k_merge_pass(const unsigned long long* __restrict__ k0, const int* __restrict__ v0, int n, int w,
                             unsigned long long* __restrict__ k1, int* __restrict__ v1) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int run = i / w, start = run * w;
    const bool left = (run & 1) == 0;
    const int ps = left ? start + w : start - w;  // partner run start
    const int pe = min(n, ps + w);
    const int base = left ? start : ps;
    const unsigned long long x = k0[i];
    int lo = min(ps, n), hi = pe;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const bool go_right = left ? (k0[mid] < x) : (k0[mid] <= x);
      if (go_right)
        lo = mid + 1;
      else
        hi = mid;
    }
    const int in_partner = ps < n ? lo - ps : 0;
    const int pos = base + (i - start) + in_partner;
    k1[pos] = x;
    v1[pos] = v0[i];
  }
}

// Renumbering of a$D_tidy_up: map[old] = new from the sorted order.
__global__ void k_map(const int* __restrict__ order, int n, int* __restrict__ map) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) map[order[i]] = i + 1;
}
__global__ void k_gather_tree(Arr o, Arr a, int dim, int nch, int nnb, const int* __restrict__ order, int used,
                              const int* __restrict__ map) {
  for (int nid = 1 + blockIdx.x * blockDim.x + threadIdx.x; nid <= used; nid += gridDim.x * blockDim.x) {
    const int k = order[nid - 1];
    a.lvl[nid] = o.lvl[k];
    a.ncell[nid] = o.ncell[k];
    a.in_use[nid] = 1;
    a.dr[nid] = o.dr[k];
    a.parent[nid] = map[o.parent[k]];
    for (int d = 0; d < dim; ++d) {
      a.ix[(size_t)nid * dim + d] = o.ix[(size_t)k * dim + d];
      a.rmin[(size_t)nid * dim + d] = o.rmin[(size_t)k * dim + d];
    }
    for (int c = 0; c < nch; ++c) a.children[(size_t)nid * nch + c] = map[o.children[(size_t)k * nch + c]];
    for (int nb = 0; nb < nnb; ++nb) {
      const int v = o.nbr[(size_t)k * nnb + nb];
      a.nbr[(size_t)nid * nnb + nb] = v > kNoBox ? map[v] : v;
    }
  }
}
__global__ void k_translate(int* __restrict__ ids, int n, const int* __restrict__ map) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ids[i] = map[ids[i]];
}

}  // namespace tdev

namespace {

int grid_of(long long n) { return (int)std::max(1LL, std::min((n + 255) / 256, 4096LL)); }

struct DBuf {
  int* p = nullptr;
  int cap = 0;
};

}  // namespace

// The device copy of a tree (see the file comment).
class DevTree {
 public:
  int device = 0;
  cudaStream_t st = nullptr;
  int dim = 2, nch = 4, nnb = 4, n_cell = 8, min_lvl = 1, lvl_limit = 30, box_limit = 0;
  int coord = 0;  // the host tree's coordinate system, carried to downloads
  int highest_lvl = 0, highest_id = 0, n_adjust = 0;
  bool ready = false;
  double dr_base = 0, r_base[3] = {0, 0, 0};
  int cap = 0;  // ids 0..cap
  tdev::Arr a{};
  struct Level {
    DBuf ids, leaves, parents;
    int n_ids = 0, n_leaves = 0, n_parents = 0;
  };
  std::vector<Level> lv;
  int* flags = nullptr;
  int flags_cap = 0;
  DBuf scan, scratch;
  unsigned long long *key0 = nullptr, *key1 = nullptr;
  int* val1 = nullptr;
  int key_cap = 0;
  int* d_small = nullptr;  // counts and sums
  int* h_small = nullptr;  // pinned copy

  ~DevTree();
  int init(const HostTree& h, int device, std::string& err);
  int adjust(const afv_ref_crit* crit, int* n_add, int* n_rm, std::string& err);
  int download(HostTree& h, std::string& err) const;

 private:
  Level& L(int l) { return lv[(size_t)(l - min_lvl)]; }
  bool ensure(DBuf& b, int n);
  bool alloc_arrays(int new_cap, tdev::Arr& out);
  void free_arrays(tdev::Arr& x);
  bool grow(int new_cap);
  int scan_list(const int* ids, int n, int prev, int mode);  // exclusive scan into `scan`; returns the total
  void split(Level& l);
  int sync_small(int n);
  void tidy_up();
};

bool DevTree::ensure(DBuf& b, int n) {
  if (n <= b.cap) return true;
  if (b.p) cudaFreeAsync(b.p, st);
  b.p = nullptr;
  b.cap = std::max(n, 2 * b.cap);
  return cudaMallocAsync((void**)&b.p, sizeof(int) * (size_t)std::max(1, b.cap), st) == cudaSuccess;
}

bool DevTree::alloc_arrays(int c, tdev::Arr& x) {
  const size_t n = (size_t)c + 1;
  x = tdev::Arr{};
  bool ok = cudaMallocAsync((void**)&x.lvl, sizeof(int) * n, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.parent, sizeof(int) * n, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.ncell, sizeof(int) * n, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.in_use, sizeof(int) * n, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.ix, sizeof(int) * n * dim, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.children, sizeof(int) * n * nch, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.nbr, sizeof(int) * n * nnb, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.dr, sizeof(double) * n, st) == cudaSuccess &&
            cudaMallocAsync((void**)&x.rmin, sizeof(double) * n * dim, st) == cudaSuccess;
  if (ok) {  // zero, as HostTree::resize does
    cudaMemsetAsync(x.lvl, 0, sizeof(int) * n, st);
    cudaMemsetAsync(x.parent, 0, sizeof(int) * n, st);
    cudaMemsetAsync(x.ncell, 0, sizeof(int) * n, st);
    cudaMemsetAsync(x.in_use, 0, sizeof(int) * n, st);
    cudaMemsetAsync(x.ix, 0, sizeof(int) * n * dim, st);
    cudaMemsetAsync(x.children, 0, sizeof(int) * n * nch, st);
    cudaMemsetAsync(x.nbr, 0, sizeof(int) * n * nnb, st);
    cudaMemsetAsync(x.dr, 0, sizeof(double) * n, st);
    cudaMemsetAsync(x.rmin, 0, sizeof(double) * n * dim, st);
  }
  return ok;
}

void DevTree::free_arrays(tdev::Arr& x) {
  for (void* p : {(void*)x.lvl, (void*)x.parent, (void*)x.ncell, (void*)x.in_use, (void*)x.ix, (void*)x.children,
                  (void*)x.nbr, (void*)x.dr, (void*)x.rmin})
    if (p) cudaFreeAsync(p, st);
  x = tdev::Arr{};
}

// Capacity for ids up to new_cap (HostTree::resize): the old arrays are copied.
bool DevTree::grow(int new_cap) {
  tdev::Arr x;
  if (!alloc_arrays(new_cap, x)) return false;
  const size_t n = (size_t)cap + 1;
  cudaMemcpyAsync(x.lvl, a.lvl, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.parent, a.parent, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.ncell, a.ncell, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.in_use, a.in_use, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.ix, a.ix, sizeof(int) * n * dim, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.children, a.children, sizeof(int) * n * nch, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.nbr, a.nbr, sizeof(int) * n * nnb, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.dr, a.dr, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(x.rmin, a.rmin, sizeof(double) * n * dim, cudaMemcpyDeviceToDevice, st);
  free_arrays(a);
  a = x;
  cap = new_cap;
  return true;
}

DevTree::~DevTree() {
  if (!st) return;
  cudaSetDevice(device);
  free_arrays(a);
  for (Level& l : lv)
    for (DBuf* b : {&l.ids, &l.leaves, &l.parents})
      if (b->p) cudaFreeAsync(b->p, st);
  for (void* p : {(void*)flags, (void*)scan.p, (void*)scratch.p, (void*)key0, (void*)key1, (void*)val1,
                  (void*)d_small})
    if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  if (h_small) cudaFreeHost(h_small);
  cudaStreamDestroy(st);
}

int DevTree::init(const HostTree& h, int dev, std::string& err) {
  if (!h.ready) return err = "tree not ready (call set_base first)", AFV_ERR_STATE;
  device = dev;
  if (cudaSetDevice(device) != cudaSuccess) return err = "cudaSetDevice failed", AFV_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
    return err = "cudaStreamCreate failed", AFV_ERR_CUDA;
  dim = h.dim;
  coord = h.coord;
  nch = h.nch;
  nnb = h.nnb;
  n_cell = h.n_cell;
  min_lvl = h.min_lvl;
  lvl_limit = h.lvl_limit;
  box_limit = h.box_limit;
  highest_lvl = h.highest_lvl;
  highest_id = h.highest_id;
  n_adjust = h.n_adjust;
  ready = h.ready;
  dr_base = h.dr_base;
  for (int d = 0; d < 3; ++d) r_base[d] = h.r_base[d];
  if (cudaMallocAsync((void**)&d_small, sizeof(int) * 8, st) != cudaSuccess ||
      cudaMallocHost((void**)&h_small, sizeof(int) * 8) != cudaSuccess)
    return err = "allocation failed", AFV_ERR_NOMEM;
  cap = std::max(h.capacity(), 1000);
  if (!alloc_arrays(cap, a)) return err = "device allocation failed", AFV_ERR_NOMEM;
  const size_t n = (size_t)h.capacity() + 1;
  cudaMemcpyAsync(a.lvl, h.lvl.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.parent, h.parent.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.ncell, h.ncell.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.in_use, h.in_use.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.ix, h.ix.data(), sizeof(int) * n * dim, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.children, h.children.data(), sizeof(int) * n * nch, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.nbr, h.neighbors.data(), sizeof(int) * n * nnb, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.dr, h.dr.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.rmin, h.r_min.data(), sizeof(double) * n * dim, cudaMemcpyHostToDevice, st);
  lv.assign(h.levels.size(), Level());
  for (size_t k = 0; k < h.levels.size(); ++k) {
    const LevelLists& s = h.levels[k];
    Level& d = lv[k];
    auto up = [&](DBuf& b, const std::vector<int>& v, int& nv) {
      nv = (int)v.size();
      if (!ensure(b, nv)) return false;
      if (nv) cudaMemcpyAsync(b.p, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, st);
      return true;
    };
    if (!up(d.ids, s.ids, d.n_ids) || !up(d.leaves, s.leaves, d.n_leaves) || !up(d.parents, s.parents, d.n_parents))
      return err = "device allocation failed", AFV_ERR_NOMEM;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return err = "upload of the tree failed", AFV_ERR_CUDA;
  return AFV_OK;
}

int DevTree::sync_small(int n) {
  cudaMemcpyAsync(h_small, d_small, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  return cudaStreamSynchronize(st) == cudaSuccess ? AFV_OK : AFV_ERR_CUDA;
}

int DevTree::scan_list(const int* ids, int n, int prev, int mode) {
  if (!ensure(scan, n)) return -1;
  if (n == 0) return 0;
  tdev::k_scan<<<1, 1024, 0, st>>>(a, nch, ids, n, flags, prev, mode, scan.p, d_small + 4);
  if (sync_small(5)) return -1;
  return h_small[4];
}

// set_leaves_parents on one level.
void DevTree::split(Level& l) {
  const int np = scan_list(l.ids.p, l.n_ids, 0, 1);
  l.n_parents = np;
  l.n_leaves = l.n_ids - np;
  ensure(l.parents, np);
  ensure(l.leaves, l.n_leaves);
  if (l.n_ids)
    tdev::k_split<<<grid_of(l.n_ids), 256, 0, st>>>(l.ids.p, l.n_ids, scan.p, a, nch, l.leaves.p, l.parents.p);
}

// a$D_tidy_up(tree, 0.5, 1000)
void DevTree::tidy_up() {
  int used = 0;
  for (int l = min_lvl; l <= highest_lvl; ++l) used += L(l).n_ids;
  const double hole_frac = 1 - used / (double)highest_id;
  const int n_clean = (int)std::lround(hole_frac * highest_id);
  if (!(hole_frac > 0.5 && n_clean >= 1000)) return;
  DBuf order;
  ensure(order, used);
  int off = 0;
  for (int l = min_lvl; l <= highest_lvl; ++l) {
    Level& v = L(l);
    const int n = v.n_ids;
    if (!n) continue;
    if (n > key_cap) {
      for (void* p : {(void*)key0, (void*)key1, (void*)val1})
        if (p) cudaFreeAsync(p, st);
      key_cap = std::max(n, 2 * key_cap);
      cudaMallocAsync((void**)&key0, sizeof(unsigned long long) * key_cap, st);
      cudaMallocAsync((void**)&key1, sizeof(unsigned long long) * key_cap, st);
      cudaMallocAsync((void**)&val1, sizeof(int) * key_cap, st);
    }
    int* v0 = order.p + off;  // the sorted ids of this level end here
    tdev::k_keys<<<grid_of(n), 256, 0, st>>>(a, dim, v.ids.p, n, key0, v0);
    unsigned long long *ka = key0, *kb = key1;
    int *va = v0, *vb = val1;
    for (int w = 1; w < n; w <<= 1) {
      tdev::k_merge_pass<<<grid_of(n), 256, 0, st>>>(ka, va, n, w, kb, vb);
      std::swap(ka, kb);
      std::swap(va, vb);
    }
    if (va != v0) cudaMemcpyAsync(v0, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
    off += n;
  }
  DBuf map;
  ensure(map, highest_id + 1);
  cudaMemsetAsync(map.p, 0, sizeof(int) * (highest_id + 1), st);
  tdev::k_map<<<grid_of(used), 256, 0, st>>>(order.p, used, map.p);
  tdev::Arr old = a, fresh;
  alloc_arrays(cap, fresh);
  // ids beyond the used range keep their old contents, except in_use
  const size_t n = (size_t)cap + 1;
  cudaMemcpyAsync(fresh.lvl, old.lvl, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.parent, old.parent, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.ncell, old.ncell, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.ix, old.ix, sizeof(int) * n * dim, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.children, old.children, sizeof(int) * n * nch, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.nbr, old.nbr, sizeof(int) * n * nnb, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.dr, old.dr, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(fresh.rmin, old.rmin, sizeof(double) * n * dim, cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(fresh.in_use, 0, sizeof(int) * n, st);
  tdev::k_gather_tree<<<grid_of(used), 256, 0, st>>>(old, fresh, dim, nch, nnb, order.p, used, map.p);
  free_arrays(old);
  a = fresh;
  // the sorted order of each level: its translated ids are increasing, i.e.
  // the old ids sorted by key, as the host builder keeps them
  off = 0;
  for (int l = min_lvl; l <= highest_lvl; ++l) {
    Level& v = L(l);
    if (!v.n_ids) continue;
    cudaMemcpyAsync(v.ids.p, order.p + off, sizeof(int) * v.n_ids, cudaMemcpyDeviceToDevice, st);
    tdev::k_translate<<<grid_of(v.n_ids), 256, 0, st>>>(v.ids.p, v.n_ids, map.p);
    off += v.n_ids;
  }
  for (int l = min_lvl; l <= highest_lvl; ++l) split(L(l));
  highest_id = used;
  cudaFreeAsync(order.p, st);
  cudaFreeAsync(map.p, st);
}

int DevTree::adjust(const afv_ref_crit* crit, int* n_add, int* n_rm, std::string& err) {
  if (!ready) return err = "tree not ready", AFV_ERR_STATE;
  if (crit->kind < AFV_REF_UNIFORM || crit->kind > AFV_REF_RANDOM_RM) return err = "unknown criterion", AFV_ERR_INVALID;
  if (crit->n_gauss > 16) return err = "at most 16 Gaussians on the device", AFV_ERR_INVALID;
  cudaSetDevice(device);
  tidy_up();
  const int prev = highest_id;
  if (prev + 1 > flags_cap) {
    if (flags) cudaFreeAsync(flags, st);
    flags_cap = std::max(prev + 1, 2 * flags_cap);
    if (cudaMallocAsync((void**)&flags, sizeof(int) * flags_cap, st) != cudaSuccess)
      return err = "device allocation failed", AFV_ERR_NOMEM;
  }
  tdev::k_fill<<<grid_of(prev + 1), 256, 0, st>>>(flags, prev + 1, tdev::kKeepRef);
  tdev::Crit c{};
  c.kind = crit->kind;
  c.lvl_max = crit->lvl_max;
  c.src_lpl = crit->src_lpl;
  c.n_gauss = crit->n_gauss;
  c.pass = n_adjust;
  c.thr = crit->thr;
  c.prob = crit->prob;
  c.seed = crit->seed;
  for (int k = 0; k < crit->n_gauss * (2 + dim) && crit->gauss; ++k) c.gauss[k] = crit->gauss[k];
  // consistent_ref_flags
  for (int l = 1; l <= highest_lvl; ++l) {
    Level& v = L(l);
    if (v.n_leaves)
      tdev::k_criterion<<<grid_of(32LL * v.n_leaves), 256, 0, st>>>(a, dim, nch, v.leaves.p, v.n_leaves, c, flags);
  }
  {
    Level& v = L(lvl_limit);
    if (v.n_ids) tdev::k_clamp<<<grid_of(v.n_ids), 256, 0, st>>>(v.ids.p, v.n_ids, flags);
  }
  for (int l = highest_lvl; l >= 1; --l) {
    Level& v = L(l);
    if (v.n_leaves) tdev::k_balance<<<grid_of(v.n_leaves), 256, 0, st>>>(a, nnb, v.leaves.p, v.n_leaves, flags);
  }
  for (int l = highest_lvl - 1; l >= 1; --l) {
    Level& v = L(l);
    if (v.n_parents) tdev::k_derefine<<<grid_of(v.n_parents), 256, 0, st>>>(a, nch, v.parents.p, v.n_parents, flags);
  }
  n_adjust++;
  cudaMemsetAsync(d_small, 0, sizeof(int) * 2, st);
  tdev::k_count<<<grid_of(prev), 256, 0, st>>>(flags, prev, d_small);
  if (sync_small(2)) return err = "refinement flags failed", AFV_ERR_CUDA;
  const int n_ref = h_small[0], n_drf = h_small[1];
  const int n_new = nch * n_ref;
  int used = 0;
  for (int l = min_lvl; l <= highest_lvl; ++l) used += L(l).n_ids;
  if ((long long)used + n_new > box_limit) {
    err = "exceeding memory limit (box_limit " + std::to_string(box_limit) + ")";
    return AFV_ERR_BUDGET;
  }
  if (prev + n_new > cap && !grow(2 * (prev + n_new))) return err = "device allocation failed", AFV_ERR_NOMEM;
  int l = 1;
  for (; l <= lvl_limit - 1; ++l) {
    Level& v = L(l);
    const int nr = scan_list(v.ids.p, v.n_ids, prev, 0);
    if (nr < 0) return err = "scan failed", AFV_ERR_CUDA;
    if (v.n_ids) {
      if (!ensure(scratch, cap + 1)) return err = "device allocation failed", AFV_ERR_NOMEM;
      tdev::k_positions<<<grid_of(v.n_ids), 256, 0, st>>>(v.ids.p, v.n_ids, scratch.p);
      tdev::k_add_remove<<<grid_of(v.n_ids), 256, 0, st>>>(a, dim, nch, nnb, v.ids.p, v.n_ids, scan.p, flags, prev,
                                                          highest_id, scratch.p);
    }
    highest_id += nch * nr;
    split(v);
    Level& u = L(l + 1);
    u.n_ids = v.n_parents * nch;
    ensure(u.ids, u.n_ids);
    if (u.n_ids) {
      tdev::k_children_of<<<grid_of(u.n_ids), 256, 0, st>>>(a, nch, v.parents.p, v.n_parents, u.ids.p);
      tdev::k_set_neighbs<<<grid_of(u.n_ids), 256, 0, st>>>(a, dim, nch, nnb, u.ids.p, u.n_ids, prev);
    }
    if (u.n_ids == 0) break;
  }
  if (l > lvl_limit - 1) l = lvl_limit;
  highest_lvl = l;
  split(L(highest_lvl + 1));
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return err = "device refinement failed", AFV_ERR_CUDA;
  if (n_add) *n_add = n_new;
  if (n_rm) *n_rm = nch * n_drf;
  return AFV_OK;
}

int DevTree::download(HostTree& h, std::string& err) const {
  cudaSetDevice(device);
  h.dim = dim;
  h.coord = coord;
  h.nch = nch;
  h.nnb = nnb;
  h.n_cell = n_cell;
  h.min_lvl = min_lvl;
  h.lvl_limit = lvl_limit;
  h.box_limit = box_limit;
  h.highest_lvl = highest_lvl;
  h.highest_id = highest_id;
  h.n_adjust = n_adjust;
  h.ready = ready;
  h.dr_base = dr_base;
  for (int d = 0; d < 3; ++d) h.r_base[d] = r_base[d];
  const size_t n = (size_t)cap + 1;
  h.lvl.assign(n, 0);
  h.parent.assign(n, 0);
  h.ncell.assign(n, 0);
  h.in_use.assign(n, 0);
  h.ix.assign(n * dim, 0);
  h.children.assign(n * nch, 0);
  h.neighbors.assign(n * nnb, 0);
  h.dr.assign(n, 0.0);
  h.r_min.assign(n * dim, 0.0);
  cudaMemcpyAsync(h.lvl.data(), a.lvl, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.parent.data(), a.parent, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.ncell.data(), a.ncell, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.in_use.data(), a.in_use, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.ix.data(), a.ix, sizeof(int) * n * dim, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.children.data(), a.children, sizeof(int) * n * nch, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.neighbors.data(), a.nbr, sizeof(int) * n * nnb, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.dr.data(), a.dr, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h.r_min.data(), a.rmin, sizeof(double) * n * dim, cudaMemcpyDeviceToHost, st);
  h.levels.assign(lv.size(), LevelLists());
  for (size_t k = 0; k < lv.size(); ++k) {
    const Level& s = lv[k];
    LevelLists& d = h.levels[k];
    d.ids.resize(s.n_ids);
    d.leaves.resize(s.n_leaves);
    d.parents.resize(s.n_parents);
    if (s.n_ids) cudaMemcpyAsync(d.ids.data(), s.ids.p, sizeof(int) * s.n_ids, cudaMemcpyDeviceToHost, st);
    if (s.n_leaves) cudaMemcpyAsync(d.leaves.data(), s.leaves.p, sizeof(int) * s.n_leaves, cudaMemcpyDeviceToHost, st);
    if (s.n_parents)
      cudaMemcpyAsync(d.parents.data(), s.parents.p, sizeof(int) * s.n_parents, cudaMemcpyDeviceToHost, st);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return err = "download of the tree failed", AFV_ERR_CUDA;
  return AFV_OK;
}

// C ABI glue (declared in afivo_gb300.h; defined here to keep DevTree local).
int dtree_create(const HostTree& h, int device, DevTree** out, std::string& err) {
  DevTree* t = new DevTree();
  int rc = t->init(h, device, err);
  if (rc) {
    delete t;
    return rc;
  }
  *out = t;
  return AFV_OK;
}
void dtree_destroy(DevTree* t) { delete t; }
int dtree_adjust(DevTree* t, const afv_ref_crit* c, int* n_add, int* n_rm, std::string& err) {
  return t->adjust(c, n_add, n_rm, err);
}
int dtree_download(const DevTree* t, HostTree& h, std::string& err) { return t->download(h, err); }
int dtree_info(const DevTree* t, int* out5) {
  out5[0] = t->highest_lvl;
  out5[1] = t->highest_id;
  out5[2] = t->n_adjust;
  int used = 0, leaves = 0;
  for (int l = t->min_lvl; l <= t->highest_lvl; ++l) {
    used += t->lv[(size_t)(l - t->min_lvl)].n_ids;
    leaves += t->lv[(size_t)(l - t->min_lvl)].n_leaves;
  }
  out5[3] = used;
  out5[4] = leaves;
  return AFV_OK;
}

}  // namespace afv
