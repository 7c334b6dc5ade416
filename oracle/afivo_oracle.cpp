// ORACLE — test infrastructure only. Nothing in the afivo_gb300 product links,
// loads or calls this file; only tests/, __graft_entry__.smoke() and the
// cpu_baseline / --impl reference legs of bench.py use it, to check the GPU
// results and as the timed CPU baseline.
//
// A C++17 + OpenMP restatement of the Afivo reference's quadtree/octree build
// and its FAS multigrid hot path. Both dimensions come from one template, the
// way the reference's m_aX_*.f90 templates are expanded (src/Makefile:28-32).
// The restatement keeps the reference's data model (1-based box ids, boxes with
// (n_cell+2)^D cell-centred storage per variable, per-level id/leaf/parent
// lists), its loop order, its OpenMP level loops and its floating-point
// evaluation order. It must be compiled with -ffp-contract=off so that no
// multiply-add is fused, matching gfortran -O2 on x86-64.
//
// Parity status: UNPINNED by reference outputs. The reference is Fortran 2008,
// there is no Fortran compiler on this machine and the reference ships no
// golden vectors for this path. The restatement is pinned instead by the
// reference's own Morton known-answer test (tests/test_morton.f90), by the
// literal topology tables of src/m_aX_t.f90:54-149, by tree invariants and by
// analytic properties of the solver (see tests/test_oracle_*.py).
//
// Deliberate deviations, all documented:
//  * All box storage is zero-initialised (the reference's `allocate` leaves it
//    undefined, src/m_aX_core.f90:352-370). The first FMG cycle reads phi on the
//    coarsest level before writing it (src/m_aX_mg.f90:520-543), so a defined
//    start value is needed for a reproducible result.
//  * box_limit uses a fixed per-box overhead in place of the compiler-specific
//    storage_size of the Fortran box type (src/m_aX_t.f90:331-341).
//  * User hooks (refinement, boundary values) are a fixed set of built-in
//    kinds, see RefCrit and BcKind below.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// src/m_aX_t.f90:17-49
constexpr int a5_rm_ref = -1;
constexpr int a5_keep_ref = 0;
constexpr int a5_do_ref = 1;
constexpr int a5_derefine = -2;
constexpr int a5_refine = 2;
constexpr int a5_no_box = 0;
constexpr int a5_init_tag = -2147483647;
constexpr int a5_bc_dirichlet = -1;
constexpr int a5_bc_neumann = -2;

// Topology tables of src/m_aX_t.f90:54-149. All of them follow from the child
// offset table a$D_child_dix (child c has offset bit d = ((c-1) >> d) & 1, x
// fastest) and from the neighbour order lowx, highx, lowy, highy[, lowz,
// highz]. tests/test_oracle_tables.py checks these functions against the
// literal reference tables.
template <int D> struct Topo {
  static constexpr int NCH = 1 << D;
  static constexpr int NNB = 2 * D;
  static int child_dix(int c, int d) { return ((c - 1) >> d) & 1; }
  static bool child_low(int c, int d) { return child_dix(c, d) == 0; }
  static int child_rev(int c, int d) { return ((c - 1) ^ (1 << d)) + 1; }
  static int neighb_dim(int nb) { return (nb - 1) / 2; }
  static bool neighb_low(int nb) { return ((nb - 1) & 1) == 0; }
  static int neighb_high_01(int nb) { return (nb - 1) & 1; }
  static int neighb_high_pm(int nb) { return ((nb - 1) & 1) ? 1 : -1; }
  static int neighb_rev(int nb) { return neighb_low(nb) ? nb + 1 : nb - 1; }
  static int neighb_dix(int nb, int d) {
    return neighb_dim(nb) == d ? neighb_high_pm(nb) : 0;
  }
  // k-th (0-based) child adjacent to neighbour direction nb (a$D_child_adj_nb)
  static int child_adj_nb(int k, int nb) {
    int d = neighb_dim(nb), h = neighb_high_01(nb), n = 0;
    for (int c = 1; c <= NCH; ++c)
      if (child_dix(c, d) == h) {
        if (n == k) return c;
        ++n;
      }
    return -1;
  }
  // a$D_ix_to_ichild, src/m_aX_t.f90:378-387
  static int ix_to_ichild(const int* ix) {
    int c = NCH;
    for (int d = 0; d < D; ++d) c -= (1 << d) * (ix[d] & 1);
    return c;
  }
};

template <int D> struct Box {
  static constexpr int NCH = 1 << D, NNB = 2 * D;
  int lvl = 0;
  bool in_use = false;
  int tag = a5_init_tag;
  int coord = 0;  // a5_xyz (0) or a5_cyl (1), src/m_aX_t.f90:42-43
  int ix[D] = {};
  int parent = 0;
  int children[NCH] = {};
  int neighbors[NNB] = {};
  int n_cell = 0;
  double dr = 0;
  double r_min[D] = {};
  int n_var = 0;
  std::vector<double> cc;  // (n_cell+2)^D per variable, x fastest
  // Face variables fx, fy[, fz] (box$D_t, src/m_aX_t.f90:153-177): per
  // variable D blocks, direction d with n_cell+1 values along d and n_cell
  // along the others, x fastest.
  int n_fc = 0;
  std::vector<double> fc;
  long long fblock() const {
    long long n = n_cell + 1;
    for (int d = 1; d < D; ++d) n *= n_cell;
    return n;
  }
  double& f_at(int ifc, int dim, int i, int j, int k) {
    const int sx = dim == 0 ? n_cell + 1 : n_cell, sy = dim == 1 ? n_cell + 1 : n_cell;
    return fc[((size_t)ifc * D + dim) * fblock() + (i - 1) + (size_t)sx * ((j - 1) + (size_t)sy * (D == 3 ? k - 1 : 0))];
  }

  int ng() const { return n_cell + 2; }
  int nvol() const {
    int n = 1;
    for (int d = 0; d < D; ++d) n *= ng();
    return n;
  }
  double& at(int i, int j, int iv) { return cc[(size_t)iv * nvol() + i + ng() * j]; }
  double& at(int i, int j, int k, int iv) {
    return cc[(size_t)iv * nvol() + i + ng() * (j + ng() * k)];
  }
  double* var(int iv) { return cc.data() + (size_t)iv * nvol(); }
};

struct Lvl {
  std::vector<int> ids, leaves, parents;
};

// Refinement criteria standing in for the user's ref_subr hook
// (src/m_aX_t.f90:231-236).
enum RefKind { REF_UNIFORM = 0, REF_GAUSS = 1, REF_RANDOM = 2, REF_RANDOM_RM = 3 };
// REF_GAUSS flags a box when any cell centre has |f| * dr**2 > thr, with f the
// sum of Gaussians (src_lpl = 0) or its Laplacian (src_lpl = 1).
struct RefCrit {
  int kind = REF_UNIFORM;
  int lvl_max = 1;
  double thr = 0;
  double prob = 0;
  uint64_t seed = 0;
  int src_lpl = 0;
  std::vector<double> gauss;  // n * (2 + D): amplitude, sigma, centre
};

// Boundary-value kinds standing in for the user's sides_bc hook
// (src/m_aX_t.f90:276-282).
enum BcKind { BC_DIRICHLET_ZERO = 0, BC_NEUMANN_ZERO = 1, BC_DIRICHLET_GAUSS = 2,
              BC_TABLE = 3 /* per (box, face) type and values, as a hook might return */ };

template <int D> struct Tree {
  static constexpr int NCH = 1 << D, NNB = 2 * D;
  bool ready = false;
  int lvl_limit = 30, box_limit = 0, highest_lvl = 0, highest_id = 0;
  int n_cell = 0, n_var_cell = 0, min_lvl = 1;
  double r_base[D] = {};
  double dr_base = 0;
  std::vector<Lvl> lvls;            // lvl = min_lvl .. lvl_limit+1
  std::vector<Box<D>> boxes;        // 1-based, boxes[0] unused
  int n_adjust = 0;                 // number of adjust_refinement calls so far
  int coord = 0;  // a5_xyz or a5_cyl (a$D_init's coord argument, core:58, 102)
  Lvl& L(int lvl) { return lvls[lvl - min_lvl]; }
  int n_boxes_capacity() const { return (int)boxes.size() - 1; }
};

// Operators of the multigrid routines (mg%box_op / box_gsrb / box_corr /
// box_rstr): the constant-coefficient Laplacian, the variable-coefficient
// lpld operators, the per-box auto dispatch (src/m_aX_mg.f90:562-706,
// 810-985), the cylindrical clpl / clpld (:1323-1443) and the level-set
// lpllsf operators (:987-1321).
enum { OP_LPL = 0, OP_LPLD = 1, OP_AUTO = 2, OP_CLPL = 3, OP_CLPLD = 4, OP_LPLLSF = 5 };
enum { MG_NORMAL_BOX = 1, MG_LSF_BOX = 2, MG_CEPS_BOX = 3, MG_VEPS_BOX = 4 };

struct MG {
  int op = OP_LPL;
  int i_eps = -1;
  int i_lsf = -1, i_bval = -1;  // level set and its boundary value (mg$D_t, mg:40-45)
  int i_phi = 0, i_rhs = 1, i_tmp = 2;
  int n_cycle_down = 2, n_cycle_up = 2, n_cycle_base = 2;
  int bc_kind = BC_DIRICHLET_ZERO;
  std::vector<double> bc_gauss;
  // BC_TABLE: per (id, face) the bc type and the offset of its face values
  // (first tangential index fastest); indexed by id * 2D + (nb - 1).
  std::vector<int> tab_type;
  std::vector<long long> tab_off;
  std::vector<double> tab_vals;
  bool initialized = false;
};

// ---------------------------------------------------------------------------
// Sources and hooks
// ---------------------------------------------------------------------------

// Sum of Gaussians a*exp(-sum(((r-c)/s)**2)), the gauss_single form of
// examples/m_gaussians.f90:64-72 with an amplitude factor.
template <int D> double gauss_src(const std::vector<double>& g, const double* r) {
  double s = 0;
  int stride = 2 + D;
  int n = (int)g.size() / stride;
  for (int k = 0; k < n; ++k) {
    const double* p = &g[(size_t)k * stride];
    double xr2 = 0;
    for (int d = 0; d < D; ++d) {
      double x = (r[d] - p[2 + d]) / p[1];
      xr2 = xr2 + x * x;
    }
    s = s + p[0] * std::exp(-xr2);
  }
  return s;
}

// Laplacian of the same sum, the gauss_lpl form of examples/m_gaussians.f90:90-102
// with an amplitude factor: a * 4/s**2 * (sum(xrel**2) - D/2) * exp(-sum(xrel**2)).
template <int D> double gauss_lpl_src(const std::vector<double>& g, const double* r) {
  double s = 0;
  int stride = 2 + D;
  int n = (int)g.size() / stride;
  for (int k = 0; k < n; ++k) {
    const double* p = &g[(size_t)k * stride];
    double xr2 = 0;
    for (int d = 0; d < D; ++d) {
      double x = (r[d] - p[2 + d]) / p[1];
      xr2 = xr2 + x * x;
    }
    s = s + p[0] * (4 / (p[1] * p[1]) * (xr2 - 0.5 * D) * std::exp(-xr2));
  }
  return s;
}

template <int D> double source_at(const std::vector<double>& g, int lpl, const double* r) {
  return lpl ? gauss_lpl_src<D>(g, r) : gauss_src<D>(g, r);
}

static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Uniform [0,1) keyed by (seed, adjust pass, lvl, ix): the same value no matter
// in which order boxes are visited, so trees are reproducible.
template <int D> double keyed_uniform(uint64_t seed, int pass, int lvl, const int* ix) {
  uint64_t h = splitmix64(seed ^ 0xA5A5A5A5ull);
  h = splitmix64(h ^ (uint64_t)(uint32_t)pass);
  h = splitmix64(h ^ (uint64_t)(uint32_t)lvl);
  for (int d = 0; d < D; ++d) h = splitmix64(h ^ (uint64_t)(uint32_t)ix[d]);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// a$D_r_cc, src/m_aX_t.f90:399-404
template <int D> void r_cc(const Box<D>& b, const int* cix, double* r) {
  for (int d = 0; d < D; ++d) r[d] = b.r_min[d] + (cix[d] - 0.5) * b.dr;
}

// Plays the role of ref_subr (e.g. examples/poisson_basic_2d.f90:105-129).
template <int D> void ref_subr(Tree<D>& t, const RefCrit& rc, int id, int& flag) {
  Box<D>& b = t.boxes[id];
  switch (rc.kind) {
    case REF_UNIFORM:
      if (b.lvl < rc.lvl_max) flag = a5_do_ref;
      break;
    case REF_GAUSS: {
      if (b.lvl >= rc.lvl_max) break;
      int nc = b.n_cell;
      double dr2 = b.dr * b.dr;
      int cix[3] = {1, 1, 1};
      int kmax = (D == 3) ? nc : 1;
      for (int k = 1; k <= kmax; ++k)
        for (int j = 1; j <= nc; ++j)
          for (int i = 1; i <= nc; ++i) {
            cix[0] = i;
            cix[1] = j;
            if (D == 3) cix[2] = k;
            double r[3];
            r_cc<D>(b, cix, r);
            double f = source_at<D>(rc.gauss, rc.src_lpl, r);
            if (std::fabs(f) * dr2 > rc.thr) {
              flag = a5_do_ref;
              return;
            }
          }
      break;
    }
    case REF_RANDOM:
    case REF_RANDOM_RM: {
      double u = keyed_uniform<D>(rc.seed, t.n_adjust, b.lvl, b.ix);
      if (u < rc.prob && b.lvl < rc.lvl_max)
        flag = a5_do_ref;
      else if (rc.kind == REF_RANDOM_RM)
        flag = a5_rm_ref;
      break;
    }
  }
}

// ---------------------------------------------------------------------------
// Tree build: src/m_aX_core.f90
// ---------------------------------------------------------------------------

template <int D> void init_box(Box<D>& b, int n_cell, int n_var) {  // core:352-370
  b.in_use = true;
  b.n_var = n_var;
  b.n_cell = n_cell;
  b.cc.assign((size_t)b.nvol() * n_var, 0.0);
}

template <int D> void clear_box(Box<D>& b) {  // core:373-384
  b.in_use = false;
  std::vector<double>().swap(b.cc);
}

// a$D_init, core:24-131
template <int D>
Tree<D>* tree_init(int n_cell, int n_var_cell, double dr, const double* r_min,
                   int lvl_limit, int n_boxes, int coarsen_to, double mem_limit_gb) {
  if (n_cell < 2 || (n_cell & 1) || n_var_cell <= 0 || n_boxes <= 0 || lvl_limit <= 0)
    return nullptr;
  auto* t = new Tree<D>();
  t->boxes.resize((size_t)n_boxes + 1);
  int min_lvl = 1;
  if (coarsen_to > 0) {
    min_lvl = 1 - (int)std::lround(std::log((double)n_cell / coarsen_to) / std::log(2.0));
    if ((1 << (1 - min_lvl)) * coarsen_to != n_cell) {
      delete t;
      return nullptr;
    }
  }
  t->min_lvl = min_lvl;
  t->lvls.assign((size_t)(lvl_limit + 1 - min_lvl + 1), Lvl());
  t->n_cell = n_cell;
  t->n_var_cell = n_var_cell;
  for (int d = 0; d < D; ++d) t->r_base[d] = r_min ? r_min[d] : 0.0;
  t->dr_base = dr;
  t->lvl_limit = lvl_limit;
  t->highest_id = 0;
  t->highest_lvl = 0;
  int nvol = 1;
  for (int d = 0; d < D; ++d) nvol *= (n_cell + 2);
  double box_bytes = 8.0 * n_var_cell * nvol + 256.0;
  t->box_limit = (int)std::lround(mem_limit_gb * 1073741824.0 / box_bytes);
  return t;
}

// get_free_ids, core:609-621
template <int D> void get_free_ids(Tree<D>& t, int n, int* ids) {
  int prev = t.highest_id;
  t.highest_id += n;
  for (int i = 0; i < n; ++i) ids[i] = prev + 1 + i;
}

// a$D_resize_box_storage, core:425-443
template <int D> void resize_box_storage(Tree<D>& t, int new_size) {
  t.boxes.resize((size_t)new_size + 1);
}

// set_leaves_parents, core:317-348
template <int D> void set_leaves_parents(std::vector<Box<D>>& boxes, Lvl& level) {
  level.parents.clear();
  level.leaves.clear();
  for (int id : level.ids) {
    if (boxes[id].children[0] != a5_no_box)
      level.parents.push_back(id);
    else
      level.leaves.push_back(id);
  }
}

// a$D_set_base, core:152-235
template <int D>
int set_base(Tree<D>& t, int n_boxes, const int* ix_list, int* nb_list) {
  using T = Topo<D>;
  constexpr int NNB = T::NNB;
  for (int i = 0; i < n_boxes * D; ++i)
    if (ix_list[i] < 1) return -1;
  if (t.highest_id > 0) return -2;
  for (int i = 1; i <= n_boxes; ++i)
    for (int nb = 1; nb <= NNB; ++nb) {
      int nb_id = nb_list[(i - 1) * NNB + nb - 1];
      if (nb_id > a5_no_box && nb_id != i) nb_list[(nb_id - 1) * NNB + T::neighb_rev(nb) - 1] = i;
    }
  for (int i = 0; i < n_boxes * NNB; ++i)
    if (nb_list[i] == a5_no_box) return -3;
  if (n_boxes > t.n_boxes_capacity()) resize_box_storage(t, n_boxes);

  for (int lvl = t.min_lvl; lvl <= 1; ++lvl) {
    Lvl& L = t.L(lvl);
    L.ids.assign(n_boxes, 0);
    get_free_ids(t, n_boxes, L.ids.data());
    int offset = L.ids[0] - 1;
    for (int i = 1; i <= n_boxes; ++i) {
      int id = L.ids[i - 1];
      Box<D>& b = t.boxes[id];
      b.lvl = lvl;
      for (int d = 0; d < D; ++d) b.ix[d] = ix_list[(i - 1) * D + d];
      b.dr = t.dr_base * std::pow(0.5, lvl - 1);
      b.coord = t.coord;
      for (int d = 0; d < D; ++d)
        b.r_min[d] = t.r_base[d] + (b.ix[d] - 1) * t.dr_base * t.n_cell;
      int nc = t.n_cell / (1 << (1 - lvl));
      b.parent = a5_no_box;
      for (int c = 0; c < T::NCH; ++c) b.children[c] = a5_no_box;
      for (int nb = 0; nb < NNB; ++nb) {
        int v = nb_list[(i - 1) * NNB + nb];
        b.neighbors[nb] = v > a5_no_box ? v + offset : v;
      }
      init_box(b, nc, t.n_var_cell);
    }
    if (lvl == 1) {
      L.leaves = L.ids;
    } else {
      L.parents = L.ids;
    }
    if (lvl > t.min_lvl) {
      Lvl& Lm = t.L(lvl - 1);
      for (int i = 0; i < n_boxes; ++i) {
        t.boxes[Lm.ids[i]].children[0] = L.ids[i];
        t.boxes[L.ids[i]].parent = Lm.ids[i];
      }
    }
  }
  t.highest_lvl = 1;
  t.ready = true;
  return 0;
}

// Morton keys, src/m_morton.f90:33-59, 96-152
static inline uint64_t bit_space_1(int a) {
  uint64_t x = (uint64_t)(int64_t)a;
  x = (x | (x << 32)) & 0x00000000ffffffffull;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
static inline int bit_despace_1(uint64_t x) {
  x = x & 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
  x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
  x = (x | (x >> 16)) & 0x00000000ffffffffull;
  return (int)(uint32_t)x;
}
static inline uint64_t bit_space_2(int a) {
  uint64_t x = (uint64_t)(int64_t)a & 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}
static inline int bit_despace_2(uint64_t x) {
  x = x & 0x1249249249249249ull;
  x = (x | (x >> 2)) & 0x10c30c30c30c30c3ull;
  x = (x | (x >> 4)) & 0x100f00f00f00f00full;
  x = (x | (x >> 8)) & 0x1f0000ff0000ffull;
  x = (x | (x >> 16)) & 0x1f00000000ffffull;
  x = (x | (x >> 32)) & 0x1fffffull;
  return (int)(uint32_t)x;
}
template <int D> uint64_t morton_from_ix(const int* ix) {
  if (D == 2) return bit_space_1(ix[0]) | (bit_space_1(ix[1]) << 1);
  return bit_space_2(ix[0]) | (bit_space_2(ix[1]) << 1) | (bit_space_2(ix[2]) << 2);
}

// morton_rank (src/m_morton.f90:155-353) is a stable merge-sort ranking. Within
// one level all keys are distinct, so every stable ranking gives the same
// permutation; a stable index sort restates it.
static void morton_rank(const std::vector<uint64_t>& keys, std::vector<int>& rank) {
  rank.resize(keys.size());
  for (size_t i = 0; i < keys.size(); ++i) rank[i] = (int)i;
  std::stable_sort(rank.begin(), rank.end(),
                   [&](int a, int b) { return keys[a] < keys[b]; });
}

// a$D_tidy_up, core:238-314
template <int D> void tidy_up(Tree<D>& t, double max_hole_frac, int n_clean_min) {
  int highest_id = t.highest_id;
  int n_used = 0;
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl) n_used += (int)t.L(lvl).ids.size();
  double hole_frac = 1 - n_used / (double)highest_id;
  int n_clean = (int)std::lround(hole_frac * highest_id);
  if (!(hole_frac > max_hole_frac && n_clean >= n_clean_min)) return;

  std::vector<Box<D>> cpy((size_t)n_used + 1);
  std::vector<int> map((size_t)highest_id + 1, 0);
  int n_stored = 0;
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl) {
    Lvl& L = t.L(lvl);
    int n = (int)L.ids.size();
    std::vector<uint64_t> keys(n);
    for (int i = 0; i < n; ++i) {
      int ixm[D];
      for (int d = 0; d < D; ++d) ixm[d] = t.boxes[L.ids[i]].ix[d] - 1;
      keys[i] = morton_from_ix<D>(ixm);
    }
    std::vector<int> rank;
    morton_rank(keys, rank);
    std::vector<int> sorted(n);
    for (int i = 0; i < n; ++i) sorted[i] = L.ids[rank[i]];
    for (int i = 0; i < n; ++i) {
      cpy[n_stored + 1 + i] = t.boxes[sorted[i]];
      map[sorted[i]] = n_stored + 1 + i;
    }
    for (int i = 0; i < n; ++i) L.ids[i] = n_stored + 1 + i;
    set_leaves_parents(cpy, L);
    n_stored += n;
  }
  for (int n = 1; n <= n_used; ++n) {
    Box<D>& b = cpy[n];
    b.parent = map[b.parent];
    for (int c = 0; c < Topo<D>::NCH; ++c) b.children[c] = map[b.children[c]];
    for (int nb = 0; nb < Topo<D>::NNB; ++nb)
      if (b.neighbors[nb] > a5_no_box) b.neighbors[nb] = map[b.neighbors[nb]];
  }
  for (int n = 1; n <= n_used; ++n) t.boxes[n] = std::move(cpy[n]);
  for (int n = n_used + 1; n <= highest_id; ++n)
    if (t.boxes[n].in_use) clear_box(t.boxes[n]);
  t.highest_id = n_used;
}

// consistent_ref_flags, core:628-725
template <int D>
int consistent_ref_flags(Tree<D>& t, std::vector<int>& ref_flags, const RefCrit& rc) {
  using T = Topo<D>;
  int lvl_limit = t.lvl_limit;
  std::fill(ref_flags.begin(), ref_flags.end(), a5_keep_ref);
#pragma omp parallel
  for (int lvl = 1; lvl <= t.highest_lvl; ++lvl) {
    Lvl& L = t.L(lvl);
#pragma omp for
    for (int i = 0; i < (int)L.leaves.size(); ++i) {
      int id = L.leaves[i];
      ref_subr(t, rc, id, ref_flags[id]);
      int p_id = t.boxes[id].parent;
      if (p_id > a5_no_box && T::ix_to_ichild(t.boxes[id].ix) == 1)
        ref_subr(t, rc, p_id, ref_flags[p_id]);
    }
  }
  for (size_t i = 1; i < ref_flags.size(); ++i)
    if (ref_flags[i] > a5_do_ref || ref_flags[i] < a5_rm_ref) return -1;

  for (int id : t.L(lvl_limit).ids)
    if (ref_flags[id] == a5_do_ref) ref_flags[id] = a5_keep_ref;

  for (int lvl = t.highest_lvl; lvl >= 1; --lvl) {
    for (int id : t.L(lvl).leaves) {
      if (ref_flags[id] > a5_keep_ref) {
        ref_flags[id] = a5_refine;
        for (int nb = 1; nb <= T::NNB; ++nb) {
          int nb_id = t.boxes[id].neighbors[nb - 1];
          if (nb_id == a5_no_box) {
            int p_id = t.boxes[id].parent;
            int p_nb_id = t.boxes[p_id].neighbors[nb - 1];
            ref_flags[p_nb_id] = a5_refine;
          }
        }
      } else if (ref_flags[id] == a5_rm_ref) {
        for (int nb = 1; nb <= T::NNB; ++nb) {
          int nb_id = t.boxes[id].neighbors[nb - 1];
          if (nb_id > a5_no_box) {
            if (t.boxes[nb_id].children[0] != a5_no_box || ref_flags[nb_id] > a5_keep_ref) {
              ref_flags[id] = a5_keep_ref;
              break;
            }
          }
        }
      }
    }
  }
  for (int lvl = t.highest_lvl - 1; lvl >= 1; --lvl) {
    for (int id : t.L(lvl).parents) {
      bool all_rm = true;
      for (int c = 0; c < T::NCH; ++c)
        if (ref_flags[t.boxes[id].children[c]] != a5_rm_ref) all_rm = false;
      if (all_rm && ref_flags[id] <= a5_keep_ref)
        ref_flags[id] = a5_derefine;
      else
        ref_flags[id] = a5_keep_ref;
    }
  }
  return 0;
}

// remove_children, core:728-749
template <int D> void remove_children(std::vector<Box<D>>& boxes, int id) {
  using T = Topo<D>;
  for (int ic = 0; ic < T::NCH; ++ic) {
    int c_id = boxes[id].children[ic];
    for (int nb = 1; nb <= T::NNB; ++nb) {
      int nb_id = boxes[c_id].neighbors[nb - 1];
      if (nb_id > a5_no_box) boxes[nb_id].neighbors[T::neighb_rev(nb) - 1] = a5_no_box;
    }
    clear_box(boxes[c_id]);
  }
  for (int ic = 0; ic < T::NCH; ++ic) boxes[id].children[ic] = a5_no_box;
}

// add_children, core:752-787
template <int D>
void add_children(std::vector<Box<D>>& boxes, int id, const int* c_ids, int n_var) {
  using T = Topo<D>;
  Box<D>& p = boxes[id];
  for (int c = 0; c < T::NCH; ++c) p.children[c] = c_ids[c];
  int c_ix_base[D];
  for (int d = 0; d < D; ++d) c_ix_base[d] = 2 * p.ix[d] - 1;
  for (int i = 1; i <= T::NCH; ++i) {
    Box<D>& c = boxes[c_ids[i - 1]];
    for (int d = 0; d < D; ++d) c.ix[d] = c_ix_base[d] + T::child_dix(i, d);
    c.lvl = p.lvl + 1;
    c.parent = id;
    c.tag = a5_init_tag;
    for (int k = 0; k < T::NCH; ++k) c.children[k] = a5_no_box;
    for (int k = 0; k < T::NNB; ++k) c.neighbors[k] = a5_no_box;
    c.dr = 0.5 * p.dr;
    c.coord = p.coord;  // core:772
    for (int d = 0; d < D; ++d)
      c.r_min[d] = p.r_min[d] + 0.5 * p.dr * T::child_dix(i, d) * p.n_cell;
    init_box(c, p.n_cell, n_var);
  }
  for (int nb = 1; nb <= T::NNB; ++nb) {
    if (p.neighbors[nb - 1] < a5_no_box) {
      for (int k = 0; k < T::NCH / 2; ++k)
        boxes[c_ids[T::child_adj_nb(k, nb) - 1]].neighbors[nb - 1] = p.neighbors[nb - 1];
    }
  }
}

// set_child_ids, core:791-808
template <int D>
void set_child_ids(const std::vector<int>& p_ids, std::vector<int>& c_ids,
                   const std::vector<Box<D>>& boxes) {
  constexpr int NCH = Topo<D>::NCH;
  c_ids.assign(p_ids.size() * NCH, 0);
  for (size_t i = 0; i < p_ids.size(); ++i)
    for (int c = 0; c < NCH; ++c) c_ids[i * NCH + c] = boxes[p_ids[i]].children[c];
}

// find_neighb_$Dd, core:404-422
template <int D> int find_neighb(const std::vector<Box<D>>& boxes, int id, int nb) {
  using T = Topo<D>;
  int p_id = boxes[id].parent;
  int c_ix = T::ix_to_ichild(boxes[id].ix);
  int d = T::neighb_dim(nb);
  if (T::child_low(c_ix, d) == T::neighb_low(nb)) p_id = boxes[p_id].neighbors[nb - 1];
  return boxes[p_id].children[T::child_rev(c_ix, d) - 1];
}

// set_neighbs_$Dd, core:387-401
template <int D> void set_neighbs(std::vector<Box<D>>& boxes, int id) {
  using T = Topo<D>;
  for (int nb = 1; nb <= T::NNB; ++nb) {
    if (boxes[id].neighbors[nb - 1] == a5_no_box) {
      int nb_id = find_neighb(boxes, id, nb);
      if (nb_id > a5_no_box) {
        boxes[id].neighbors[nb - 1] = nb_id;
        boxes[nb_id].neighbors[T::neighb_rev(nb) - 1] = id;
      }
    }
  }
}

// a$D_adjust_refinement, core:452-541 (ref_info reduced to n_add / n_rm,
// set_ref_info core:544-605)
template <int D>
int adjust_refinement(Tree<D>& t, const RefCrit& rc, int* n_add, int* n_rm) {
  using T = Topo<D>;
  if (!t.ready) return -1;
  tidy_up(t, 0.5, 1000);
  int highest_id_prev = t.highest_id;
  std::vector<int> ref_flags((size_t)highest_id_prev + 1, a5_keep_ref);
  if (consistent_ref_flags(t, ref_flags, rc) != 0) return -2;
  t.n_adjust++;
  int n_ref = 0, n_drf = 0;
  for (int id = 1; id <= highest_id_prev; ++id) {
    if (ref_flags[id] == a5_refine) n_ref++;
    if (ref_flags[id] == a5_derefine) n_drf++;
  }
  int num_new_boxes = T::NCH * n_ref;
  int n_used = 0;
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl) n_used += (int)t.L(lvl).ids.size();
  if (n_used + num_new_boxes > t.box_limit) return -3;
  int highest_id_req = highest_id_prev + num_new_boxes;
  if (highest_id_req > t.n_boxes_capacity()) resize_box_storage(t, 2 * highest_id_req);

  int lvl;
  for (lvl = 1; lvl <= t.lvl_limit - 1; ++lvl) {
    Lvl& L = t.L(lvl);
    for (size_t i = 0; i < L.ids.size(); ++i) {
      int id = L.ids[i];
      if (id > highest_id_prev) continue;
      if (ref_flags[id] == a5_refine) {
        int c_ids[T::NCH];
        get_free_ids(t, T::NCH, c_ids);
        add_children(t.boxes, id, c_ids, t.n_var_cell);
      } else if (ref_flags[id] == a5_derefine) {
        remove_children(t.boxes, id);
      }
    }
    set_leaves_parents(t.boxes, L);
    set_child_ids(L.parents, t.L(lvl + 1).ids, t.boxes);
    for (int id : t.L(lvl + 1).ids)
      if (id > highest_id_prev) set_neighbs(t.boxes, id);
    if (t.L(lvl + 1).ids.empty()) break;
  }
  if (lvl > t.lvl_limit - 1) lvl = t.lvl_limit;
  t.highest_lvl = lvl;
  set_leaves_parents(t.boxes, t.L(t.highest_lvl + 1));
  if (n_add) *n_add = T::NCH * n_ref;
  if (n_rm) *n_rm = T::NCH * n_drf;
  return 0;
}

// ---------------------------------------------------------------------------
// Grid operators: src/m_aX_gc.f90, m_aX_prolong.f90, m_aX_restrict.f90,
// m_aX_utils.f90
// ---------------------------------------------------------------------------

// a$D_get_child_offset, src/m_aX_t.f90:362-374 (without the nb argument)
template <int D> void child_offset(const Box<D>& c, int* off) {
  for (int d = 0; d < D; ++d) off[d] = c.lvl > 1 ? (((c.ix[d] - 1) & 1) * (c.n_cell >> 1)) : 0;
}

// sides_from_nb, gc:381-415
template <int D> void sides_from_nb(Box<D>& b, Box<D>& nbb, int nb, int iv) {
  int nc = b.n_cell;
  if constexpr (D == 2) {
    for (int n = 1; n <= nc; ++n) {
      switch (nb) {
        case 1: b.at(0, n, iv) = nbb.at(nc, n, iv); break;
        case 2: b.at(nc + 1, n, iv) = nbb.at(1, n, iv); break;
        case 3: b.at(n, 0, iv) = nbb.at(n, nc, iv); break;
        case 4: b.at(n, nc + 1, iv) = nbb.at(n, 1, iv); break;
      }
    }
  } else {
    for (int m = 1; m <= nc; ++m)
      for (int n = 1; n <= nc; ++n) {
        switch (nb) {
          case 1: b.at(0, n, m, iv) = nbb.at(nc, n, m, iv); break;
          case 2: b.at(nc + 1, n, m, iv) = nbb.at(1, n, m, iv); break;
          case 3: b.at(n, 0, m, iv) = nbb.at(n, nc, m, iv); break;
          case 4: b.at(n, nc + 1, m, iv) = nbb.at(n, 1, m, iv); break;
          case 5: b.at(n, m, 0, iv) = nbb.at(n, m, nc, iv); break;
          case 6: b.at(n, m, nc + 1, iv) = nbb.at(n, m, 1, iv); break;
        }
      }
  }
}

// Ghost-face cell (a, b) of face nb (a, b run over 1..nc in the two (one)
// face directions, x before y before z).
template <int D> double& face_ghost(Box<D>& b, int nb, int a, int c) {
  int nc = b.n_cell;
  if constexpr (D == 2) {
    switch (nb) {
      case 1: return b.at(0, a, 0);
      case 2: return b.at(nc + 1, a, 0);
      case 3: return b.at(a, 0, 0);
      default: return b.at(a, nc + 1, 0);
    }
  } else {
    switch (nb) {
      case 1: return b.at(0, a, c, 0);
      case 2: return b.at(nc + 1, a, c, 0);
      case 3: return b.at(a, 0, c, 0);
      case 4: return b.at(a, nc + 1, c, 0);
      case 5: return b.at(a, c, 0, 0);
      default: return b.at(a, c, nc + 1, 0);
    }
  }
}

// The user's sides_bc hook: writes the boundary value b into the ghost face and
// returns the type (a$D_bc_dirichlet_zero / a$D_bc_neumann_zero, gc:361-378;
// the position-dependent form of examples/poisson_basic_2d.f90:167-203).
template <int D> int sides_bc(Box<D>& b, int id, int nb, int iv, const MG& mg) {
  using T = Topo<D>;
  int nc = b.n_cell;
  int vol = b.nvol();
  int bc_type = (mg.bc_kind == BC_NEUMANN_ZERO) ? a5_bc_neumann : a5_bc_dirichlet;
  size_t tk = (size_t)id * T::NNB + (nb - 1);
  if (mg.bc_kind == BC_TABLE) bc_type = mg.tab_type[tk];
  int cmax = (D == 3) ? nc : 1;
  for (int c = 1; c <= cmax; ++c)
    for (int a = 1; a <= nc; ++a) {
      double val = 0.0;
      if (mg.bc_kind == BC_TABLE) {
        val = mg.tab_vals[mg.tab_off[tk] + (size_t)(c - 1) * nc + (a - 1)];
      } else if (mg.bc_kind == BC_DIRICHLET_GAUSS) {
        // Face centre: a$D_rr_cc with 0.5 or nc+0.5 in the normal direction.
        double rr[3];
        int d = T::neighb_dim(nb);
        int k = 0;
        int tang[2] = {a, c};
        for (int e = 0; e < D; ++e) {
          double cix;
          if (e == d)
            cix = T::neighb_low(nb) ? 0.5 : nc + 0.5;
          else
            cix = (double)tang[k++];
          rr[e] = b.r_min[e] + (cix - 0.5) * b.dr;
        }
        val = gauss_src<D>(mg.bc_gauss, rr);
      }
      (&face_ghost<D>(b, nb, a, c))[(size_t)iv * vol] = val;
    }
  return bc_type;
}

// bc_to_gc, gc:71-132
template <int D> void bc_to_gc(Box<D>& b, int nb, int iv, int bc_type) {
  using T = Topo<D>;
  int nc = b.n_cell;
  double c1, c2;
  if (bc_type == a5_bc_dirichlet) {
    c1 = -1;
    c2 = 2;
  } else {
    c1 = 1;
    c2 = b.dr * T::neighb_high_pm(nb);
  }
  if constexpr (D == 2) {
    for (int n = 1; n <= nc; ++n) {
      switch (nb) {
        case 1: b.at(0, n, iv) = c2 * b.at(0, n, iv) + c1 * b.at(1, n, iv); break;
        case 2: b.at(nc + 1, n, iv) = c2 * b.at(nc + 1, n, iv) + c1 * b.at(nc, n, iv); break;
        case 3: b.at(n, 0, iv) = c2 * b.at(n, 0, iv) + c1 * b.at(n, 1, iv); break;
        case 4: b.at(n, nc + 1, iv) = c2 * b.at(n, nc + 1, iv) + c1 * b.at(n, nc, iv); break;
      }
    }
  } else {
    for (int m = 1; m <= nc; ++m)
      for (int n = 1; n <= nc; ++n) {
        switch (nb) {
          case 1: b.at(0, n, m, iv) = c2 * b.at(0, n, m, iv) + c1 * b.at(1, n, m, iv); break;
          case 2: b.at(nc + 1, n, m, iv) = c2 * b.at(nc + 1, n, m, iv) + c1 * b.at(nc, n, m, iv); break;
          case 3: b.at(n, 0, m, iv) = c2 * b.at(n, 0, m, iv) + c1 * b.at(n, 1, m, iv); break;
          case 4: b.at(n, nc + 1, m, iv) = c2 * b.at(n, nc + 1, m, iv) + c1 * b.at(n, nc, m, iv); break;
          case 5: b.at(n, m, 0, iv) = c2 * b.at(n, m, 0, iv) + c1 * b.at(n, m, 1, iv); break;
          case 6: b.at(n, m, nc + 1, iv) = c2 * b.at(n, m, nc + 1, iv) + c1 * b.at(n, m, nc, iv); break;
        }
      }
  }
}

// a$D_prolong0 over a partial range (add = false), prolong:39-108
template <int D>
void prolong0(Box<D>& p, Box<D>& c, int iv, const int* lo, const int* hi) {
  int off[D];
  child_offset(c, off);
  if constexpr (D == 2) {
    for (int j = lo[1]; j <= hi[1]; ++j) {
      int j_c1 = off[1] + ((j + 1) >> 1);
      for (int i = lo[0]; i <= hi[0]; ++i) {
        int i_c1 = off[0] + ((i + 1) >> 1);
        c.at(i, j, iv) = p.at(i_c1, j_c1, iv);
      }
    }
  } else {
    for (int k = lo[2]; k <= hi[2]; ++k) {
      int k_c1 = off[2] + ((k + 1) >> 1);
      for (int j = lo[1]; j <= hi[1]; ++j) {
        int j_c1 = off[1] + ((j + 1) >> 1);
        for (int i = lo[0]; i <= hi[0]; ++i) {
          int i_c1 = off[0] + ((i + 1) >> 1);
          c.at(i, j, k, iv) = p.at(i_c1, j_c1, k_c1, iv);
        }
      }
    }
  }
}

// a$D_gc_prolong0, gc:135-151
template <int D> void gc_prolong0(Tree<D>& t, int id, int nb, int iv) {
  using T = Topo<D>;
  Box<D>& b = t.boxes[id];
  int lo[D], hi[D];
  for (int d = 0; d < D; ++d) {
    lo[d] = 1;
    hi[d] = b.n_cell;
  }
  int nd = T::neighb_dim(nb);
  lo[nd] = T::neighb_high_01(nb) * (b.n_cell + 1);
  hi[nd] = lo[nd];
  prolong0(t.boxes[b.parent], b, iv, lo, hi);
}

// mg$D_sides_rb, src/m_aX_mg.f90:262-350
template <int D> void sides_rb(Tree<D>& t, int id, int nb, int iv) {
  using T = Topo<D>;
  Box<D>& b = t.boxes[id];
  int nc = b.n_cell;
  int ix, dix;
  if (T::neighb_low(nb)) {
    ix = 1;
    dix = 1;
  } else {
    ix = nc;
    dix = -1;
  }
  gc_prolong0(t, id, nb, iv);
  if constexpr (D == 2) {
    if (T::neighb_dim(nb) == 0) {
      int i = ix, di = dix;
      for (int j = 1; j <= nc; ++j) {
        int dj = -1 + 2 * (j & 1);
        b.at(i - di, j, iv) = 0.5 * b.at(i - di, j, iv) + b.at(i, j, iv) -
                              0.25 * (b.at(i + di, j, iv) + b.at(i, j + dj, iv));
      }
    } else {
      int j = ix, dj = dix;
      for (int i = 1; i <= nc; ++i) {
        int di = -1 + 2 * (i & 1);
        b.at(i, j - dj, iv) = 0.5 * b.at(i, j - dj, iv) + b.at(i, j, iv) -
                              0.25 * (b.at(i + di, j, iv) + b.at(i, j + dj, iv));
      }
    }
  } else {
    switch (T::neighb_dim(nb)) {
      case 0: {
        int i = ix, di = dix;
        for (int k = 1; k <= nc; ++k) {
          int dk = -1 + 2 * (k & 1);
          for (int j = 1; j <= nc; ++j) {
            int dj = -1 + 2 * (j & 1);
            b.at(i - di, j, k, iv) = 0.5 * b.at(i - di, j, k, iv) + 0.75 * b.at(i, j, k, iv) -
                                     0.25 * b.at(i + di, j + dj, k + dk, iv);
          }
        }
        break;
      }
      case 1: {
        int j = ix, dj = dix;
        for (int k = 1; k <= nc; ++k) {
          int dk = -1 + 2 * (k & 1);
          for (int i = 1; i <= nc; ++i) {
            int di = -1 + 2 * (i & 1);
            b.at(i, j - dj, k, iv) = 0.5 * b.at(i, j - dj, k, iv) + 0.75 * b.at(i, j, k, iv) -
                                     0.25 * b.at(i + di, j + dj, k + dk, iv);
          }
        }
        break;
      }
      default: {
        int k = ix, dk = dix;
        for (int j = 1; j <= nc; ++j) {
          int dj = -1 + 2 * (j & 1);
          for (int i = 1; i <= nc; ++i) {
            int di = -1 + 2 * (i & 1);
            b.at(i, j, k - dk, iv) = 0.5 * b.at(i, j, k - dk, iv) + 0.75 * b.at(i, j, k, iv) -
                                     0.25 * b.at(i + di, j + dj, k + dk, iv);
          }
        }
        break;
      }
    }
  }
}

// a$D_gc_box with mg%sides_rb = mg$D_sides_rb and mg%sides_bc, gc:50-69
template <int D> void gc_box(Tree<D>& t, int id, int iv, const MG& mg) {
  using T = Topo<D>;
  for (int nb = 1; nb <= T::NNB; ++nb) {
    int nb_id = t.boxes[id].neighbors[nb - 1];
    if (nb_id > a5_no_box) {
      sides_from_nb(t.boxes[id], t.boxes[nb_id], nb, iv);
    } else if (nb_id == a5_no_box) {
      sides_rb(t, id, nb, iv);
    } else {
      int bc_type = sides_bc(t.boxes[id], id, nb, iv, mg);
      bc_to_gc(t.boxes[id], nb, iv, bc_type);
    }
  }
}

// a$D_prolong2 (add = .true.), prolong:243-348
template <int D> void prolong2_add(Box<D>& p, Box<D>& c, int iv, int ivc) {
  int hnc = c.n_cell >> 1;
  int off[D];
  child_offset(c, off);
  if constexpr (D == 2) {
    for (int j = 1; j <= hnc; ++j) {
      int j_c = j + off[1], j_f = 2 * j - 1;
      for (int i = 1; i <= hnc; ++i) {
        int i_c = i + off[0], i_f = 2 * i - 1;
        double f0 = p.at(i_c, j_c, iv);
        double fx = 0.125 * (p.at(i_c + 1, j_c, iv) - p.at(i_c - 1, j_c, iv));
        double fy = 0.125 * (p.at(i_c, j_c + 1, iv) - p.at(i_c, j_c - 1, iv));
        double fxx = 0.03125 * (p.at(i_c - 1, j_c, iv) - 2 * f0 + p.at(i_c + 1, j_c, iv));
        double fyy = 0.03125 * (p.at(i_c, j_c - 1, iv) - 2 * f0 + p.at(i_c, j_c + 1, iv));
        double f2 = fxx + fyy;
        c.at(i_f, j_f, ivc) = f0 - fx - fy + f2 + c.at(i_f, j_f, ivc);
        c.at(i_f + 1, j_f, ivc) = f0 + fx - fy + f2 + c.at(i_f + 1, j_f, ivc);
        c.at(i_f, j_f + 1, ivc) = f0 - fx + fy + f2 + c.at(i_f, j_f + 1, ivc);
        c.at(i_f + 1, j_f + 1, ivc) = f0 + fx + fy + f2 + c.at(i_f + 1, j_f + 1, ivc);
      }
    }
  } else {
    for (int k = 1; k <= hnc; ++k) {
      int k_c = k + off[2], k_f = 2 * k - 1;
      for (int j = 1; j <= hnc; ++j) {
        int j_c = j + off[1], j_f = 2 * j - 1;
        for (int i = 1; i <= hnc; ++i) {
          int i_c = i + off[0], i_f = 2 * i - 1;
          double f0 = p.at(i_c, j_c, k_c, iv);
          double fx = 0.125 * (p.at(i_c + 1, j_c, k_c, iv) - p.at(i_c - 1, j_c, k_c, iv));
          double fy = 0.125 * (p.at(i_c, j_c + 1, k_c, iv) - p.at(i_c, j_c - 1, k_c, iv));
          double fz = 0.125 * (p.at(i_c, j_c, k_c + 1, iv) - p.at(i_c, j_c, k_c - 1, iv));
          double fxx = 0.03125 * (p.at(i_c - 1, j_c, k_c, iv) - 2 * f0 + p.at(i_c + 1, j_c, k_c, iv));
          double fyy = 0.03125 * (p.at(i_c, j_c - 1, k_c, iv) - 2 * f0 + p.at(i_c, j_c + 1, k_c, iv));
          double fzz = 0.03125 * (p.at(i_c, j_c, k_c - 1, iv) - 2 * f0 + p.at(i_c, j_c, k_c + 1, iv));
          double f2 = fxx + fyy + fzz;
          c.at(i_f, j_f, k_f, ivc) = f0 - fx - fy - fz + f2 + c.at(i_f, j_f, k_f, ivc);
          c.at(i_f + 1, j_f, k_f, ivc) = f0 + fx - fy - fz + f2 + c.at(i_f + 1, j_f, k_f, ivc);
          c.at(i_f, j_f + 1, k_f, ivc) = f0 - fx + fy - fz + f2 + c.at(i_f, j_f + 1, k_f, ivc);
          c.at(i_f + 1, j_f + 1, k_f, ivc) = f0 + fx + fy - fz + f2 + c.at(i_f + 1, j_f + 1, k_f, ivc);
          c.at(i_f, j_f, k_f + 1, ivc) = f0 - fx - fy + fz + f2 + c.at(i_f, j_f, k_f + 1, ivc);
          c.at(i_f + 1, j_f, k_f + 1, ivc) = f0 + fx - fy + fz + f2 + c.at(i_f + 1, j_f, k_f + 1, ivc);
          c.at(i_f, j_f + 1, k_f + 1, ivc) = f0 - fx + fy + fz + f2 + c.at(i_f, j_f + 1, k_f + 1, ivc);
          c.at(i_f + 1, j_f + 1, k_f + 1, ivc) = f0 + fx + fy + fz + f2 + c.at(i_f + 1, j_f + 1, k_f + 1, ivc);
        }
      }
    }
  }
}

// a2_cyl_child_weights, src/m_aX_t.f90:516-528: the inner and outer
// children's weights at cell index i of a box with lower radius r_min0 and
// cell size dr (the cell centre's radius, a2_cyl_radius_cc, :508-514).
inline void cyl_child_weights(double r_min0, double dr, int i, double& inner, double& outer) {
  const double r = r_min0 + (i - 0.5) * dr;
  const double tmp = 0.25 * dr / r;
  inner = 1 - tmp;
  outer = 1 + tmp;
}

// a$D_restrict_box, restrict:67-132. The Fortran sum() of a 2^D section
// accumulates column-major from zero. In cylindrical trees the inner and
// outer pairs take the parent's weights at index i (:90-103; the index
// within the quadrant, as the reference passes it).
template <int D> void restrict_box(Box<D>& c, Box<D>& p, int iv) {
  int hnc = c.n_cell >> 1;
  int off[D];
  child_offset(c, off);
  if (D == 2 && p.coord == 1) {
    for (int j = 1; j <= hnc; ++j) {
      int j_c = off[1] + j, j_f = 2 * j - 1;
      for (int i = 1; i <= hnc; ++i) {
        int i_c = off[0] + i, i_f = 2 * i - 1;
        double w1, w2;
        cyl_child_weights(p.r_min[0], p.dr, i, w1, w2);
        double s1 = 0.0, s2 = 0.0;
        s1 = s1 + c.at(i_f, j_f, 0, iv);
        s1 = s1 + c.at(i_f, j_f + 1, 0, iv);
        s2 = s2 + c.at(i_f + 1, j_f, 0, iv);
        s2 = s2 + c.at(i_f + 1, j_f + 1, 0, iv);
        p.at(i_c, j_c, 0, iv) = 0.25 * (w1 * s1 + w2 * s2);
      }
    }
    return;
  }
  if constexpr (D == 2) {
    for (int j = 1; j <= hnc; ++j) {
      int j_c = off[1] + j, j_f = 2 * j - 1;
      for (int i = 1; i <= hnc; ++i) {
        int i_c = off[0] + i, i_f = 2 * i - 1;
        double s = 0.0;
        s = s + c.at(i_f, j_f, iv);
        s = s + c.at(i_f + 1, j_f, iv);
        s = s + c.at(i_f, j_f + 1, iv);
        s = s + c.at(i_f + 1, j_f + 1, iv);
        p.at(i_c, j_c, iv) = 0.25 * s;
      }
    }
  } else {
    for (int k = 1; k <= hnc; ++k) {
      int k_c = off[2] + k, k_f = 2 * k - 1;
      for (int j = 1; j <= hnc; ++j) {
        int j_c = off[1] + j, j_f = 2 * j - 1;
        for (int i = 1; i <= hnc; ++i) {
          int i_c = off[0] + i, i_f = 2 * i - 1;
          double s = 0.0;
          for (int kk = 0; kk < 2; ++kk)
            for (int jj = 0; jj < 2; ++jj)
              for (int ii = 0; ii < 2; ++ii) s = s + c.at(i_f + ii, j_f + jj, k_f + kk, iv);
          p.at(i_c, j_c, k_c, iv) = 0.125 * s;
        }
      }
    }
  }
}

// mg$D_box_gsrb_lpl, mg:718-760
template <int D> void box_gsrb_lpl(Box<D>& b, int redblack_cntr, const MG& mg) {
  double dx2 = b.dr * b.dr;
  int nc = b.n_cell;
  int ip = mg.i_phi, ir = mg.i_rhs;
  if constexpr (D == 2) {
    for (int j = 1; j <= nc; ++j) {
      int i0 = 2 - ((redblack_cntr ^ j) & 1);
      for (int i = i0; i <= nc; i += 2)
        b.at(i, j, ip) = 0.25 * (b.at(i + 1, j, ip) + b.at(i - 1, j, ip) + b.at(i, j + 1, ip) +
                                 b.at(i, j - 1, ip) - dx2 * b.at(i, j, ir));
    }
  } else {
    const double sixth = 1 / 6.0;
    for (int k = 1; k <= nc; ++k)
      for (int j = 1; j <= nc; ++j) {
        int i0 = 2 - ((redblack_cntr ^ (k + j)) & 1);
        for (int i = i0; i <= nc; i += 2)
          b.at(i, j, k, ip) =
              sixth * (b.at(i + 1, j, k, ip) + b.at(i - 1, j, k, ip) + b.at(i, j + 1, k, ip) +
                       b.at(i, j - 1, k, ip) + b.at(i, j, k + 1, ip) + b.at(i, j, k - 1, ip) -
                       dx2 * b.at(i, j, k, ir));
      }
  }
}

// mg$D_box_lpl, mg:763-797
template <int D> void box_lpl(Box<D>& b, int i_out, const MG& mg) {
  int nc = b.n_cell;
  double inv_dr_sq = 1 / (b.dr * b.dr);
  int ip = mg.i_phi;
  if constexpr (D == 2) {
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i)
        b.at(i, j, i_out) = inv_dr_sq * (b.at(i - 1, j, ip) + b.at(i + 1, j, ip) + b.at(i, j - 1, ip) +
                                         b.at(i, j + 1, ip) - 4 * b.at(i, j, ip));
  } else {
    for (int k = 1; k <= nc; ++k)
      for (int j = 1; j <= nc; ++j)
        for (int i = 1; i <= nc; ++i)
          b.at(i, j, k, i_out) =
              inv_dr_sq * (b.at(i - 1, j, k, ip) + b.at(i + 1, j, k, ip) + b.at(i, j - 1, k, ip) +
                           b.at(i, j + 1, k, ip) + b.at(i, j, k - 1, ip) + b.at(i, j, k + 1, ip) -
                           6 * b.at(i, j, k, ip));
  }
}

// mg$D_set_box_tag (mg:672-706): min and max of lsf and eps over the whole
// box, ghost cells included. Returns false where the reference stops (a box
// that would take two tags).
template <int D> bool set_box_tag(Box<D>& b, const MG& mg) {
  bool is_lsf = false, is_eps = false, is_deps = false;
  auto minmax = [&](int iv, double& a, double& c) {
    const double* e = b.var(iv);
    a = e[0];
    c = e[0];
    for (int n = 0; n < b.nvol(); ++n) {
      a = std::min(a, e[n]);
      c = std::max(c, e[n]);
    }
  };
  if (mg.i_lsf != -1) {
    double a, c;
    minmax(mg.i_lsf, a, c);
    is_lsf = a * c < 0;
  }
  if (mg.i_eps != -1) {
    double a, c;
    minmax(mg.i_eps, a, c);
    is_deps = c > a;
    if (!is_deps) is_eps = (a < 1 || a > 1);
  }
  b.tag = MG_NORMAL_BOX;
  if (is_lsf) b.tag = MG_LSF_BOX;
  if (is_eps) b.tag = MG_CEPS_BOX;
  if (is_deps) b.tag = MG_VEPS_BOX;
  return (int)is_lsf + (int)is_eps + (int)is_deps <= 1;
}

// Neighbour values of cell (i,j[,k]) in the reference's order (i-1, i+1,
// j-1, j+1[, k-1, k+1]).
template <int D> void nb_vals(Box<D>& b, int iv, int i, int j, int k, double* out) {
  if constexpr (D == 2) {
    out[0] = b.at(i - 1, j, iv);
    out[1] = b.at(i + 1, j, iv);
    out[2] = b.at(i, j - 1, iv);
    out[3] = b.at(i, j + 1, iv);
  } else {
    out[0] = b.at(i - 1, j, k, iv);
    out[1] = b.at(i + 1, j, k, iv);
    out[2] = b.at(i, j - 1, k, iv);
    out[3] = b.at(i, j + 1, k, iv);
    out[4] = b.at(i, j, k - 1, iv);
    out[5] = b.at(i, j, k + 1, iv);
  }
}

// mg$D_box_gsrb_lpld, mg:810-859
template <int D> void box_gsrb_lpld(Box<D>& b, int redblack_cntr, const MG& mg) {
  const double dx2 = b.dr * b.dr;
  const int nc = b.n_cell, ip = mg.i_phi, ie = mg.i_eps, ir = mg.i_rhs;
  const int kmax = D == 3 ? nc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= nc; ++j) {
      const int i0 = 2 - ((redblack_cntr ^ (D == 3 ? k + j : j)) & 1);
      for (int i = i0; i <= nc; i += 2) {
        double u[6], a[6], c[6];
        const double a0 = D == 2 ? b.at(i, j, ie) : b.at(i, j, k, ie);
        nb_vals<D>(b, ip, i, j, k, u);
        nb_vals<D>(b, ie, i, j, k, a);
        for (int n = 0; n < 2 * D; ++n) c[n] = 2 * a0 * a[n] / (a0 + a[n]);
        double scu = 0.0, sc = 0.0;
        for (int n = 0; n < 2 * D; ++n) scu = scu + c[n] * u[n];
        for (int n = 0; n < 2 * D; ++n) sc = sc + c[n];
        double& o = D == 2 ? b.at(i, j, ip) : b.at(i, j, k, ip);
        o = (scu - dx2 * (D == 2 ? b.at(i, j, ir) : b.at(i, j, k, ir))) / sc;
      }
    }
}

// mg$D_box_lpld, mg:861-905
template <int D> void box_lpld(Box<D>& b, int i_out, const MG& mg) {
  const int nc = b.n_cell, ip = mg.i_phi, ie = mg.i_eps;
  const double inv_dr_sq = 1 / (b.dr * b.dr);
  const int kmax = D == 3 ? nc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        double u[6], a[6];
        const double u0 = D == 2 ? b.at(i, j, ip) : b.at(i, j, k, ip);
        const double a0 = D == 2 ? b.at(i, j, ie) : b.at(i, j, k, ie);
        nb_vals<D>(b, ip, i, j, k, u);
        nb_vals<D>(b, ie, i, j, k, a);
        double s = 0.0;
        for (int n = 0; n < 2 * D; ++n) s = s + a0 * a[n] / (a0 + a[n]) * (u[n] - u0);
        (D == 2 ? b.at(i, j, i_out) : b.at(i, j, k, i_out)) = inv_dr_sq * 2 * s;
      }
}

// mg$D_box_corr_lpld, mg:907-985
template <int D> void box_corr_lpld(Box<D>& p, Box<D>& c, const MG& mg) {
  const int nc = c.n_cell, ip = mg.i_phi, it = mg.i_tmp, ie = mg.i_eps;
  int off[D];
  child_offset(c, off);
  const double third = 1 / 3.0;
  const int kmax = D == 3 ? nc : 1;
  for (int k = 1; k <= kmax; ++k) {
    const int k_c1 = D == 3 ? off[D - 1] + ((k + 1) >> 1) : 0;
    const int k_c2 = k_c1 + 1 - 2 * (k & 1);
    for (int j = 1; j <= nc; ++j) {
      const int j_c1 = off[1] + ((j + 1) >> 1), j_c2 = j_c1 + 1 - 2 * (j & 1);
      for (int i = 1; i <= nc; ++i) {
        const int i_c1 = off[0] + ((i + 1) >> 1), i_c2 = i_c1 + 1 - 2 * (i & 1);
        if constexpr (D == 2) {
          const double u0 = p.at(i_c1, j_c1, it), a0 = p.at(i_c1, j_c1, ie);
          const double u[2] = {p.at(i_c2, j_c1, it), p.at(i_c1, j_c2, it)};
          const double a[2] = {p.at(i_c2, j_c1, ie), p.at(i_c1, j_c2, ie)};
          double s = 0.0;
          for (int n = 0; n < 2; ++n) s = s + (a0 * u0 + a[n] * u[n]) / (a0 + a[n]);
          c.at(i, j, ip) = c.at(i, j, ip) + 0.5 * s;
        } else {
          const double u0 = p.at(i_c1, j_c1, k_c1, it), a0 = p.at(i_c1, j_c1, k_c1, ie);
          const double u[3] = {p.at(i_c2, j_c1, k_c1, it), p.at(i_c1, j_c2, k_c1, it), p.at(i_c1, j_c1, k_c2, it)};
          const double a[3] = {p.at(i_c2, j_c1, k_c1, ie), p.at(i_c1, j_c2, k_c1, ie), p.at(i_c1, j_c1, k_c2, ie)};
          double s = 0.0;
          for (int n = 0; n < 3; ++n) s = s + (a0 * u0 + a[n] * (1.5 * u[n] - 0.5 * u0)) / (a0 + a[n]);
          c.at(i, j, k, ip) = c.at(i, j, k, ip) + third * s;
        }
      }
    }
  }
}

// mg2_box_gsrb_clpl / mg2_box_clpl / mg2_box_clpld / mg2_box_gsrb_clpld,
// mg:1323-1443 (2-D only): the cylindrical operators, radial factors
// rfac = [i+ioff-1, i+ioff] / (i+ioff-0.5) with ioff = (ix(1)-1) * nc.
template <int D> void box_gsrb_clpl(Box<D>& b, int redblack_cntr, const MG& mg) {
  if constexpr (D == 2) {
    const double dx2 = b.dr * b.dr;
    const int nc = b.n_cell, ip = mg.i_phi, ir = mg.i_rhs, ioff = (b.ix[0] - 1) * nc;
    for (int j = 1; j <= nc; ++j) {
      const int i0 = 2 - ((redblack_cntr ^ j) & 1);
      for (int i = i0; i <= nc; i += 2) {
        const double r1 = (i + ioff - 1) / (i + ioff - 0.5), r2 = (i + ioff) / (i + ioff - 0.5);
        b.at(i, j, ip) = 0.25 * (r1 * b.at(i - 1, j, ip) + r2 * b.at(i + 1, j, ip) + b.at(i, j + 1, ip) +
                                 b.at(i, j - 1, ip) - dx2 * b.at(i, j, ir));
      }
    }
  }
}
template <int D> void box_clpl(Box<D>& b, int i_out, const MG& mg) {
  if constexpr (D == 2) {
    const double inv_dr_sq = 1 / (b.dr * b.dr);
    const int nc = b.n_cell, ip = mg.i_phi, ioff = (b.ix[0] - 1) * nc;
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        const double r1 = (i + ioff - 1) / (i + ioff - 0.5), r2 = (i + ioff) / (i + ioff - 0.5);
        b.at(i, j, i_out) = (r1 * b.at(i - 1, j, ip) + r2 * b.at(i + 1, j, ip) + b.at(i, j - 1, ip) +
                             b.at(i, j + 1, ip) - 4 * b.at(i, j, ip)) *
                            inv_dr_sq;
      }
  }
}
template <int D> void box_clpld(Box<D>& b, int i_out, const MG& mg) {
  if constexpr (D == 2) {
    const double inv_dr_sq = 1 / (b.dr * b.dr);
    const int nc = b.n_cell, ip = mg.i_phi, ie = mg.i_eps, ioff = (b.ix[0] - 1) * nc;
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        const double rfac[4] = {(i + ioff - 1) / (i + ioff - 0.5), (i + ioff) / (i + ioff - 0.5), 1, 1};
        double u[4], a[4];
        const double u0 = b.at(i, j, ip), a0 = b.at(i, j, ie);
        nb_vals<D>(b, ip, i, j, 0, u);
        nb_vals<D>(b, ie, i, j, 0, a);
        double s = 0.0;
        for (int n = 0; n < 4; ++n) s = s + rfac[n] * a0 * a[n] / (a0 + a[n]) * (u[n] - u0);
        b.at(i, j, i_out) = inv_dr_sq * 2 * s;
      }
  }
}
template <int D> void box_gsrb_clpld(Box<D>& b, int redblack_cntr, const MG& mg) {
  if constexpr (D == 2) {
    const double dx2 = b.dr * b.dr;
    const int nc = b.n_cell, ip = mg.i_phi, ie = mg.i_eps, ir = mg.i_rhs, ioff = (b.ix[0] - 1) * nc;
    for (int j = 1; j <= nc; ++j) {
      const int i0 = 2 - ((redblack_cntr ^ j) & 1);
      for (int i = i0; i <= nc; i += 2) {
        const double rfac[4] = {(i + ioff - 1) / (i + ioff - 0.5), (i + ioff) / (i + ioff - 0.5), 1, 1};
        double u[4], a[4], c[4];
        const double a0 = b.at(i, j, ie);
        nb_vals<D>(b, ip, i, j, 0, u);
        nb_vals<D>(b, ie, i, j, 0, a);
        for (int n = 0; n < 4; ++n) c[n] = 2 * a0 * a[n] / (a0 + a[n]);
        double s1 = 0.0, s2 = 0.0;
        for (int n = 0; n < 4; ++n) s1 = s1 + c[n] * rfac[n] * u[n];
        for (int n = 0; n < 4; ++n) s2 = s2 + c[n] * rfac[n];
        b.at(i, j, ip) = (s1 - dx2 * b.at(i, j, ir)) / s2;
      }
    }
  }
}

// lsf_dist_val, mg:993-1019: distance (0..1) to a neighbour and the value
// there, or at the interface between when the level set changes sign.
// a and b hold (level set, value, boundary value).
inline void lsf_dist_val(const double* a, const double* b, double& dist, double& val) {
  const double lsf_a = a[0], lsf_b = b[0];
  if (lsf_a * lsf_b < 0) {
    dist = lsf_a / (lsf_a - lsf_b);
    val = a[2] * (1 - dist) + b[2] * dist;
  } else {
    dist = 1;
    val = b[1];
  }
}
template <int D> void lsf_triple(Box<D>& b, const MG& mg, int i, int j, int k, double* v) {
  const int iv[3] = {mg.i_lsf, mg.i_phi, mg.i_bval};
  for (int n = 0; n < 3; ++n) v[n] = D == 2 ? b.at(i, j, iv[n]) : b.at(i, j, k, iv[n]);
}
// The 2D neighbours' distances and values (i-1, i+1, j-1, j+1[, k-1, k+1]).
template <int D> void lsf_stencil(Box<D>& b, const MG& mg, int i, int j, int k, double* dd, double* val) {
  double va[3], vb[3];
  lsf_triple<D>(b, mg, i, j, k, va);
  const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
  for (int n = 0; n < 2 * D; ++n) {
    lsf_triple<D>(b, mg, i + di[n], j + dj[n], k + dk[n], vb);
    lsf_dist_val(va, vb, dd[n], val[n]);
  }
}

// mg$D_box_gsrb_lpllsf, mg:1102-1181
template <int D> void box_gsrb_lpllsf(Box<D>& b, int redblack_cntr, const MG& mg) {
  const double dx2 = b.dr * b.dr;
  const int nc = b.n_cell, ip = mg.i_phi, ir = mg.i_rhs;
  const int kmax = D == 3 ? nc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= nc; ++j) {
      const int i0 = 2 - ((redblack_cntr ^ (D == 3 ? k + j : j)) & 1);
      for (int i = i0; i <= nc; i += 2) {
        double dd[6], val[6];
        lsf_stencil<D>(b, mg, i, j, k, dd, val);
        if constexpr (D == 2) {
          double prod = 1;
          for (int n = 0; n < 4; ++n) prod = prod * dd[n];
          b.at(i, j, ip) = 1 / (dd[0] * dd[1] + dd[2] * dd[3]) *
                           ((dd[1] * val[0] + dd[0] * val[1]) * dd[2] * dd[3] / (dd[0] + dd[1]) +
                            (dd[3] * val[2] + dd[2] * val[3]) * dd[0] * dd[1] / (dd[2] + dd[3]) -
                            0.5 * prod * dx2 * b.at(i, j, ir));
        } else {
          b.at(i, j, k, ip) =
              1 / (1 / (dd[0] * dd[1]) + 1 / (dd[2] * dd[3]) + 1 / (dd[4] * dd[5])) *
              ((dd[1] * val[0] + dd[0] * val[1]) / ((dd[0] + dd[1]) * dd[0] * dd[1]) +
               (dd[3] * val[2] + dd[2] * val[3]) / ((dd[2] + dd[3]) * dd[2] * dd[3]) +
               (dd[5] * val[4] + dd[4] * val[5]) / ((dd[4] + dd[5]) * dd[4] * dd[5]) - 0.5 * dx2 * b.at(i, j, k, ir));
        }
      }
    }
}

// mg$D_box_lpllsf, mg:1184-1253
template <int D> void box_lpllsf(Box<D>& b, int i_out, const MG& mg) {
  const double inv_dr_sq = 1 / (b.dr * b.dr);
  const int nc = b.n_cell, ip = mg.i_phi;
  const int kmax = D == 3 ? nc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        double dd[6], val[6];
        lsf_stencil<D>(b, mg, i, j, k, dd, val);
        const double f0 = D == 2 ? b.at(i, j, ip) : b.at(i, j, k, ip);
        double s = (dd[1] * val[0] + dd[0] * val[1] - (dd[0] + dd[1]) * f0) / ((dd[0] + dd[1]) * dd[0] * dd[1]) +
                   (dd[3] * val[2] + dd[2] * val[3] - (dd[2] + dd[3]) * f0) / ((dd[2] + dd[3]) * dd[2] * dd[3]);
        if constexpr (D == 3)
          s = s + (dd[5] * val[4] + dd[4] * val[5] - (dd[4] + dd[5]) * f0) / ((dd[4] + dd[5]) * dd[4] * dd[5]);
        (D == 2 ? b.at(i, j, i_out) : b.at(i, j, k, i_out)) = 2 * inv_dr_sq * s;
      }
}

// mg$D_box_corr_lpllsf, mg:1021-1099
template <int D> void box_corr_lpllsf(Box<D>& p, Box<D>& c, const MG& mg) {
  const int nc = c.n_cell, ip = mg.i_phi, icr = mg.i_tmp, il = mg.i_lsf;
  int off[D];
  child_offset(c, off);
  const int kmax = D == 3 ? nc : 1;
  for (int k = 1; k <= kmax; ++k) {
    const int k_c1 = D == 3 ? off[D - 1] + ((k + 1) >> 1) : 0, k_c2 = k_c1 + 1 - 2 * (k & 1);
    for (int j = 1; j <= nc; ++j) {
      const int j_c1 = off[1] + ((j + 1) >> 1), j_c2 = j_c1 + 1 - 2 * (j & 1);
      for (int i = 1; i <= nc; ++i) {
        const int i_c1 = off[0] + ((i + 1) >> 1), i_c2 = i_c1 + 1 - 2 * (i & 1);
        auto P = [&](int a, int b, int e, int iv) { return D == 2 ? p.at(a, b, iv) : p.at(a, b, e, iv); };
        double va[3], vb[3], dist[4], val[4];
        va[0] = D == 2 ? c.at(i, j, il) : c.at(i, j, k, il);
        va[1] = D == 2 ? c.at(i, j, icr) : c.at(i, j, k, icr);
        va[2] = 0.0;
        vb[2] = 0.0;
        const int pts[4][3] = {{i_c1, j_c1, k_c1}, {i_c2, j_c1, k_c1}, {i_c1, j_c2, k_c1}, {i_c1, j_c1, k_c2}};
        for (int n = 0; n <= D; ++n) {
          vb[0] = P(pts[n][0], pts[n][1], pts[n][2], il);
          vb[1] = P(pts[n][0], pts[n][1], pts[n][2], icr);
          lsf_dist_val(va, vb, dist[n], val[n]);
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
        for (int n = 0; n <= D; ++n) s1 = s1 + cw[n] * val[n];
        for (int n = 0; n <= D; ++n) s2 = s2 + cw[n];
        double& o = D == 2 ? c.at(i, j, ip) : c.at(i, j, k, ip);
        o = o + s1 / s2;
      }
    }
  }
}

// mg$D_box_rstr_lpllsf, mg:1256-1320: children on the parent's side of the
// interface only; 1 / n_ch is an integer division in the reference.
template <int D> void box_rstr_lpllsf(Box<D>& c, Box<D>& p, int iv, const MG& mg) {
  const int hnc = c.n_cell >> 1, il = mg.i_lsf, nch = 1 << D;
  int off[D];
  child_offset(c, off);
  const int kmax = D == 3 ? hnc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= hnc; ++j)
      for (int i = 1; i <= hnc; ++i) {
        const int i_c = off[0] + i, j_c = off[1] + j, k_c = D == 3 ? off[D - 1] + k : 0;
        const int i_f = 2 * i - 1, j_f = 2 * j - 1, k_f = 2 * k - 1;
        const double lp = D == 2 ? p.at(i_c, j_c, il) : p.at(i_c, j_c, k_c, il);
        int n_ch = 0;
        double sm = 0.0, sa = 0.0;
        for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
          for (int jj = 0; jj < 2; ++jj)
            for (int ii = 0; ii < 2; ++ii) {
              const double lc = D == 2 ? c.at(i_f + ii, j_f + jj, il) : c.at(i_f + ii, j_f + jj, k_f + kk, il);
              const double v = D == 2 ? c.at(i_f + ii, j_f + jj, iv) : c.at(i_f + ii, j_f + jj, k_f + kk, iv);
              sa = sa + v;
              if (lp * lc > 0) {
                ++n_ch;
                sm = sm + v;
              }
            }
        double& o = D == 2 ? p.at(i_c, j_c, iv) : p.at(i_c, j_c, k_c, iv);
        if (n_ch < nch && n_ch > 0)
          o = (double)(1 / n_ch) * sm;
        else
          o = (D == 2 ? 0.25 : 0.125) * sa;
      }
}

// The operator of a box as the driver calls mg%box_gsrb / box_op / box_corr
// / box_rstr: the fixed choice, or mg$D_auto_* by the box's tag (mg:562-669;
// the tag is taken at first use).
enum { K_LPL = 0, K_LPLD = 1, K_CLPL = 2, K_CLPLD = 3, K_LSF = 4 };
template <int D> int box_kind(Box<D>& b, const MG& mg) {
  switch (mg.op) {
    case OP_LPL: return K_LPL;
    case OP_LPLD: return K_LPLD;
    case OP_CLPL: return K_CLPL;
    case OP_CLPLD: return K_CLPLD;
    case OP_LPLLSF: return K_LSF;
  }
  if (b.tag == a5_init_tag) set_box_tag<D>(b, mg);
  const bool cyl = D == 2 && b.coord == 1;
  switch (b.tag) {
    case MG_NORMAL_BOX: return cyl ? K_CLPL : K_LPL;
    case MG_LSF_BOX: return K_LSF;
    default: return cyl ? K_CLPLD : K_LPLD;
  }
}

// Interior / full-array helpers, utils:262-352
template <int D> void interior_for(Box<D>& b, int iv_a, int iv_b, int mode) {
  // mode 0: b = a - b ; mode 1: b = a (interior only)
  int nc = b.n_cell;
  int kmax = (D == 3) ? nc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        double* pa;
        double* pb;
        if constexpr (D == 2) {
          pa = &b.at(i, j, iv_a);
          pb = &b.at(i, j, iv_b);
        } else {
          pa = &b.at(i, j, k, iv_a);
          pb = &b.at(i, j, k, iv_b);
        }
        if (mode == 0)
          *pb = *pa - *pb;
        else
          *pb = *pa;
      }
}

// residual_box, mg:545-559
template <int D> void box_op(Box<D>& b, int i_out, const MG& mg) {
  switch (box_kind<D>(b, mg)) {
    case K_LPL: box_lpl<D>(b, i_out, mg); break;
    case K_LPLD: box_lpld<D>(b, i_out, mg); break;
    case K_CLPL: box_clpl<D>(b, i_out, mg); break;
    case K_CLPLD: box_clpld<D>(b, i_out, mg); break;
    default: box_lpllsf<D>(b, i_out, mg); break;
  }
}
template <int D> void box_gsrb(Box<D>& b, int n, const MG& mg) {
  switch (box_kind<D>(b, mg)) {
    case K_LPL: box_gsrb_lpl<D>(b, n, mg); break;
    case K_LPLD: box_gsrb_lpld<D>(b, n, mg); break;
    case K_CLPL: box_gsrb_clpl<D>(b, n, mg); break;
    case K_CLPLD: box_gsrb_clpld<D>(b, n, mg); break;
    default: box_gsrb_lpllsf<D>(b, n, mg); break;
  }
}
// mg%box_corr: mg$D_auto_corr (mg:645-669) chooses by the child's tag; the
// cylindrical operators take the Cartesian corrections
template <int D> void box_corr(Box<D>& p, Box<D>& c, const MG& mg) {
  switch (box_kind<D>(c, mg)) {
    case K_LPL:
    case K_CLPL: prolong2_add<D>(p, c, mg.i_tmp, mg.i_phi); break;
    case K_LSF: box_corr_lpllsf<D>(p, c, mg); break;
    default: box_corr_lpld<D>(p, c, mg); break;
  }
}
// mg%box_rstr: mg$D_auto_rstr (mg:625-642) by the child's tag, lpllsf's
// masked average for level-set boxes, a$D_restrict_box otherwise
template <int D> void box_rstr(Box<D>& c, Box<D>& p, int iv, const MG& mg) {
  if (box_kind<D>(c, mg) == K_LSF)
    box_rstr_lpllsf<D>(c, p, iv, mg);
  else
    restrict_box<D>(c, p, iv);
}

template <int D> void residual_box(Box<D>& b, const MG& mg) {
  box_op(b, mg.i_tmp, mg);
  interior_for(b, mg.i_rhs, mg.i_tmp, 0);
}

template <int D> void box_clear_cc(Box<D>& b, int iv) {  // utils:262-270
  double* v = b.var(iv);
  std::fill(v, v + b.nvol(), 0.0);
}
template <int D> void box_add_cc(Box<D>& b, int iv_from, int iv_to) {  // utils:273-281
  double* f = b.var(iv_from);
  double* t = b.var(iv_to);
  for (int n = 0; n < b.nvol(); ++n) t[n] = t[n] + f[n];
}
template <int D> void box_copy_cc(Box<D>& b, int iv_from, int iv_to) {  // utils:331-339
  double* f = b.var(iv_from);
  double* t = b.var(iv_to);
  for (int n = 0; n < b.nvol(); ++n) t[n] = f[n];
}

// ---------------------------------------------------------------------------
// Multigrid: src/m_aX_mg.f90
// ---------------------------------------------------------------------------

template <int D> void fill_gc_phi(Tree<D>& t, const std::vector<int>& ids, const MG& mg) {
#pragma omp parallel for
  for (int i = 0; i < (int)ids.size(); ++i) gc_box(t, ids[i], mg.i_phi, mg);
}

template <int D> void correct_children(Tree<D>& t, const std::vector<int>& ids, const MG& mg) {
#pragma omp parallel for
  for (int i = 0; i < (int)ids.size(); ++i) {
    int id = ids[i];
    Box<D>& p = t.boxes[id];
    double* ph = p.var(mg.i_phi);
    double* tm = p.var(mg.i_tmp);
    for (int n = 0; n < p.nvol(); ++n) tm[n] = ph[n] - tm[n];
    for (int ic = 0; ic < Topo<D>::NCH; ++ic) {
      int c_id = p.children[ic];
      if (c_id == a5_no_box) continue;
      box_corr<D>(p, t.boxes[c_id], mg);
    }
  }
}

template <int D>
void gsrb_boxes(Tree<D>& t, const std::vector<int>& ids, const MG& mg, int n_cycle) {
#pragma omp parallel
  for (int n = 1; n <= 2 * n_cycle; ++n) {
#pragma omp for
    for (int i = 0; i < (int)ids.size(); ++i) box_gsrb<D>(t.boxes[ids[i]], n, mg);
#pragma omp for
    for (int i = 0; i < (int)ids.size(); ++i) gc_box(t, ids[i], mg.i_phi, mg);
  }
}

// update_coarse, mg:424-480
template <int D> void update_coarse(Tree<D>& t, int lvl, const MG& mg) {
  const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp parallel for
  for (int i = 0; i < (int)ids.size(); ++i) {
    int id = ids[i];
    Box<D>& b = t.boxes[id];
    int p_id = b.parent;
    std::vector<double> save(t.boxes[id].var(mg.i_tmp), t.boxes[id].var(mg.i_tmp) + b.nvol());
    residual_box(b, mg);
    box_rstr<D>(b, t.boxes[p_id], mg.i_tmp, mg);
    box_rstr<D>(b, t.boxes[p_id], mg.i_phi, mg);
    // restore the interior of tmp (the ghost cells of tmp are not touched above)
    std::copy(save.begin(), save.end(), b.var(mg.i_tmp));
  }
  fill_gc_phi(t, t.L(lvl - 1).ids, mg);
  const std::vector<int>& par = t.L(lvl - 1).parents;
#pragma omp parallel for
  for (int i = 0; i < (int)par.size(); ++i) {
    Box<D>& p = t.boxes[par[i]];
    box_op<D>(p, mg.i_rhs, mg);
    box_add_cc(p, mg.i_tmp, mg.i_rhs);
    box_copy_cc(p, mg.i_phi, mg.i_tmp);
  }
}

// set_coarse_phi_rhs, mg:484-517
template <int D> void set_coarse_phi_rhs(Tree<D>& t, int lvl, const MG& mg) {
  if (lvl == t.highest_lvl) fill_gc_phi(t, t.L(lvl).ids, mg);
  const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp parallel for
  for (int i = 0; i < (int)ids.size(); ++i) {
    Box<D>& b = t.boxes[ids[i]];
    residual_box(b, mg);
    box_rstr<D>(b, t.boxes[b.parent], mg.i_tmp, mg);
    box_rstr<D>(b, t.boxes[b.parent], mg.i_phi, mg);
  }
  fill_gc_phi(t, t.L(lvl - 1).ids, mg);
  const std::vector<int>& par = t.L(lvl - 1).parents;
#pragma omp parallel for
  for (int i = 0; i < (int)par.size(); ++i) {
    Box<D>& p = t.boxes[par[i]];
    box_op<D>(p, mg.i_rhs, mg);
    box_add_cc(p, mg.i_tmp, mg.i_rhs);
  }
}

// init_phi_rhs, mg:520-543
template <int D> void init_phi_rhs(Tree<D>& t, const MG& mg) {
#pragma omp parallel
  for (int lvl = t.highest_lvl; lvl >= t.min_lvl + 1; --lvl) {
    const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp for
    for (int i = 0; i < (int)ids.size(); ++i) {
      Box<D>& b = t.boxes[ids[i]];
      box_clear_cc(b, mg.i_phi);
      box_rstr<D>(b, t.boxes[b.parent], mg.i_rhs, mg);
    }
  }
}

// mg$D_fas_vcycle, mg:208-255
template <int D> void fas_vcycle(Tree<D>& t, const MG& mg, int highest_lvl, bool set_residual) {
  int min_lvl = t.min_lvl;
  for (int lvl = highest_lvl; lvl >= min_lvl + 1; --lvl) {
    gsrb_boxes(t, t.L(lvl).ids, mg, mg.n_cycle_down);
    update_coarse(t, lvl, mg);
  }
  gsrb_boxes(t, t.L(min_lvl).ids, mg, mg.n_cycle_base);
  for (int lvl = min_lvl + 1; lvl <= highest_lvl; ++lvl) {
    correct_children(t, t.L(lvl - 1).parents, mg);
    fill_gc_phi(t, t.L(lvl).ids, mg);
    gsrb_boxes(t, t.L(lvl).ids, mg, mg.n_cycle_up);
  }
  if (set_residual) {
#pragma omp parallel
    for (int lvl = min_lvl; lvl <= highest_lvl; ++lvl) {
      const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp for
      for (int i = 0; i < (int)ids.size(); ++i) residual_box(t.boxes[ids[i]], mg);
    }
  }
}

// mg$D_fas_fmg, mg:164-203
template <int D> void fas_fmg(Tree<D>& t, const MG& mg, bool set_residual, bool have_guess) {
  int min_lvl = t.min_lvl;
  if (have_guess) {
    for (int lvl = t.highest_lvl; lvl >= min_lvl + 1; --lvl) set_coarse_phi_rhs(t, lvl, mg);
  } else {
    init_phi_rhs(t, mg);
  }
  for (int lvl = min_lvl; lvl <= t.highest_lvl; ++lvl) {
    const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp parallel for
    for (int i = 0; i < (int)ids.size(); ++i) box_copy_cc(t.boxes[ids[i]], mg.i_phi, mg.i_tmp);
    if (lvl > min_lvl) {
      correct_children(t, t.L(lvl - 1).parents, mg);
      fill_gc_phi(t, t.L(lvl).ids, mg);
    }
    fas_vcycle(t, mg, lvl, set_residual && lvl == t.highest_lvl);
  }
}

// a$D_tree_max_cc / a$D_tree_min_cc over leaves, utils:468-571
template <int D> double tree_max_cc(Tree<D>& t, int iv, bool want_max) {
  double best = want_max ? -1.7976931348623157e308 : 1.7976931348623157e308;
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl) {
    const std::vector<int>& lv = t.L(lvl).leaves;
    for (int id : lv) {
      Box<D>& b = t.boxes[id];
      int nc = b.n_cell;
      int kmax = (D == 3) ? nc : 1;
      for (int k = 1; k <= kmax; ++k)
        for (int j = 1; j <= nc; ++j)
          for (int i = 1; i <= nc; ++i) {
            double v = (D == 2) ? b.at(i, j, iv) : b.at(i, j, k, iv);
            if (want_max ? (v > best) : (v < best)) best = v;
          }
    }
  }
  return best;
}

// Mean of a variable over leaf interiors, weighted by cell volume (used for the
// singular periodic problem, where the solution is fixed up to a constant).
template <int D> double leaf_mean(Tree<D>& t, int iv) {
  double s = 0, w = 0;
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl)
    for (int id : t.L(lvl).leaves) {
      Box<D>& b = t.boxes[id];
      int nc = b.n_cell;
      double vol = 1;
      for (int d = 0; d < D; ++d) vol *= b.dr;
      int kmax = (D == 3) ? nc : 1;
      for (int k = 1; k <= kmax; ++k)
        for (int j = 1; j <= nc; ++j)
          for (int i = 1; i <= nc; ++i) {
            s += vol * ((D == 2) ? b.at(i, j, iv) : b.at(i, j, k, iv));
            w += vol;
          }
    }
  return s / w;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C ABI used by the tests and the CPU baseline (ctypes).
// ---------------------------------------------------------------------------
using namespace orc;

// ---------------------------------------------------------------------------
// General ghost-cell, transfer and output routines used by codes other than
// the multigrid solver: src/m_aX_prolong.f90, m_aX_restrict.f90:21-64,
// m_aX_gc.f90:28-358, 420-634, m_aX_core.f90:811-945, m_aX_io.f90:115-310,
// m_vtk.f90.
// ---------------------------------------------------------------------------

// n_var_cell / n_var_face of a$D_init (core:24-131) grown on a built tree:
// n_cc more cell variables after the existing ones and n_fc face variables,
// zero-initialised.
template <int D> void add_vars(Tree<D>& t, int n_cc, int n_fc) {
  t.n_var_cell += n_cc;
  for (size_t id = 1; id < t.boxes.size(); ++id) {
    Box<D>& b = t.boxes[id];
    if (!b.in_use) continue;
    b.n_var += n_cc;
    b.cc.resize((size_t)b.nvol() * b.n_var, 0.0);
    if (n_fc) {
      b.n_fc = n_fc;
      b.fc.assign((size_t)n_fc * D * b.fblock(), 0.0);
    }
  }
}

// a$D_prolong0 / a$D_prolong1 / a$D_prolong2 of a whole child (prolong:39-348)
template <int D> void prolong_box(Box<D>& p, Box<D>& c, int iv, int ivc, int order, bool add) {
  const int nc = c.n_cell, hnc = nc >> 1;
  int off[D];
  child_offset(c, off);
  if (order == 0) {
    const int kmax = D == 3 ? nc : 1;
    for (int k = 1; k <= kmax; ++k) {
      const int k_c1 = D == 3 ? off[D - 1] + ((k + 1) >> 1) : 0;
      for (int j = 1; j <= nc; ++j) {
        const int j_c1 = off[1] + ((j + 1) >> 1);
        for (int i = 1; i <= nc; ++i) {
          const int i_c1 = off[0] + ((i + 1) >> 1);
          double& o = D == 2 ? c.at(i, j, ivc) : c.at(i, j, k, ivc);
          const double v = D == 2 ? p.at(i_c1, j_c1, iv) : p.at(i_c1, j_c1, k_c1, iv);
          o = add ? o + v : v;
        }
      }
    }
    return;
  }
  if (!add) {  // box_c%cc(1:nc, 1:nc[, 1:nc], ivc) = 0
    const int kmax = D == 3 ? nc : 1;
    for (int k = 1; k <= kmax; ++k)
      for (int j = 1; j <= nc; ++j)
        for (int i = 1; i <= nc; ++i) (D == 2 ? c.at(i, j, ivc) : c.at(i, j, k, ivc)) = 0;
  }
  if (order == 2) {  // onto the zeroed interior unless add, as the reference does
    prolong2_add<D>(p, c, iv, ivc);
    return;
  }
  // order 1: 2-1-1 (2D) and 1-1-1-1 (3D) interpolation, prolong:129-222
  if constexpr (D == 2) {
    for (int j = 1; j <= hnc; ++j) {
      const int j_c = j + off[1], j_f = 2 * j - 1;
      for (int i = 1; i <= hnc; ++i) {
        const int i_c = i + off[0], i_f = 2 * i - 1;
        const double f0 = 0.5 * p.at(i_c, j_c, iv);
        const double flx = 0.25 * p.at(i_c - 1, j_c, iv);
        const double fhx = 0.25 * p.at(i_c + 1, j_c, iv);
        const double fly = 0.25 * p.at(i_c, j_c - 1, iv);
        const double fhy = 0.25 * p.at(i_c, j_c + 1, iv);
        c.at(i_f, j_f, ivc) = f0 + flx + fly + c.at(i_f, j_f, ivc);
        c.at(i_f + 1, j_f, ivc) = f0 + fhx + fly + c.at(i_f + 1, j_f, ivc);
        c.at(i_f, j_f + 1, ivc) = f0 + flx + fhy + c.at(i_f, j_f + 1, ivc);
        c.at(i_f + 1, j_f + 1, ivc) = f0 + fhx + fhy + c.at(i_f + 1, j_f + 1, ivc);
      }
    }
  } else {
    for (int k = 1; k <= hnc; ++k) {
      const int k_c = k + off[2], k_f = 2 * k - 1;
      for (int j = 1; j <= hnc; ++j) {
        const int j_c = j + off[1], j_f = 2 * j - 1;
        for (int i = 1; i <= hnc; ++i) {
          const int i_c = i + off[0], i_f = 2 * i - 1;
          const double f0 = 0.25 * p.at(i_c, j_c, k_c, iv);
          const double flx = 0.25 * p.at(i_c - 1, j_c, k_c, iv);
          const double fhx = 0.25 * p.at(i_c + 1, j_c, k_c, iv);
          const double fly = 0.25 * p.at(i_c, j_c - 1, k_c, iv);
          const double fhy = 0.25 * p.at(i_c, j_c + 1, k_c, iv);
          const double flz = 0.25 * p.at(i_c, j_c, k_c - 1, iv);
          const double fhz = 0.25 * p.at(i_c, j_c, k_c + 1, iv);
          c.at(i_f, j_f, k_f, ivc) = f0 + flx + fly + flz + c.at(i_f, j_f, k_f, ivc);
          c.at(i_f + 1, j_f, k_f, ivc) = f0 + fhx + fly + flz + c.at(i_f + 1, j_f, k_f, ivc);
          c.at(i_f, j_f + 1, k_f, ivc) = f0 + flx + fhy + flz + c.at(i_f, j_f + 1, k_f, ivc);
          c.at(i_f + 1, j_f + 1, k_f, ivc) = f0 + fhx + fhy + flz + c.at(i_f + 1, j_f + 1, k_f, ivc);
          c.at(i_f, j_f, k_f + 1, ivc) = f0 + flx + fly + fhz + c.at(i_f, j_f, k_f + 1, ivc);
          c.at(i_f + 1, j_f, k_f + 1, ivc) = f0 + fhx + fly + fhz + c.at(i_f + 1, j_f, k_f + 1, ivc);
          c.at(i_f, j_f + 1, k_f + 1, ivc) = f0 + flx + fhy + fhz + c.at(i_f, j_f + 1, k_f + 1, ivc);
          c.at(i_f + 1, j_f + 1, k_f + 1, ivc) = f0 + fhx + fhy + fhz + c.at(i_f + 1, j_f + 1, k_f + 1, ivc);
        }
      }
    }
  }
}

// a$D_prolong{0,1,2}_from (prolong:22-37, 112-127, 226-241) on the parents of a level
template <int D> void prolong_from_level(Tree<D>& t, int lvl, int iv, int ivc, int order, bool add) {
  using T = Topo<D>;
  for (int id : t.L(lvl).parents)
    for (int i_c = 0; i_c < T::NCH; ++i_c) {
      const int c_id = t.boxes[id].children[i_c];
      if (c_id == a5_no_box) continue;
      prolong_box<D>(t.boxes[id], t.boxes[c_id], iv, ivc, order, add);
    }
}

// a$D_restrict_box with iv_to (restrict:67-132)
template <int D> void restrict_box_to(Box<D>& c, Box<D>& p, int iv, int ivt) {
  const int hnc = c.n_cell >> 1;
  int off[D];
  child_offset(c, off);
  if (D == 2 && p.coord == 1) {  // cylindrical branch, restrict:90-103
    for (int j = 1; j <= hnc; ++j)
      for (int i = 1; i <= hnc; ++i) {
        const int i_f = 2 * i - 1, j_f = 2 * j - 1;
        double w1, w2;
        cyl_child_weights(p.r_min[0], p.dr, i, w1, w2);
        double s1 = 0.0, s2 = 0.0;
        s1 = s1 + c.at(i_f, j_f, 0, iv);
        s1 = s1 + c.at(i_f, j_f + 1, 0, iv);
        s2 = s2 + c.at(i_f + 1, j_f, 0, iv);
        s2 = s2 + c.at(i_f + 1, j_f + 1, 0, iv);
        p.at(off[0] + i, off[1] + j, 0, ivt) = 0.25 * (w1 * s1 + w2 * s2);
      }
    return;
  }
  const int kmax = D == 3 ? hnc : 1;
  for (int k = 1; k <= kmax; ++k)
    for (int j = 1; j <= hnc; ++j)
      for (int i = 1; i <= hnc; ++i) {
        const int i_f = 2 * i - 1, j_f = 2 * j - 1, k_f = 2 * k - 1;
        double s = 0.0;
        if constexpr (D == 2) {
          s = s + c.at(i_f, j_f, iv);
          s = s + c.at(i_f + 1, j_f, iv);
          s = s + c.at(i_f, j_f + 1, iv);
          s = s + c.at(i_f + 1, j_f + 1, iv);
          p.at(off[0] + i, off[1] + j, ivt) = 0.25 * s;
        } else {
          for (int kk = 0; kk < 2; ++kk)
            for (int jj = 0; jj < 2; ++jj)
              for (int ii = 0; ii < 2; ++ii) s = s + c.at(i_f + ii, j_f + jj, k_f + kk, iv);
          p.at(off[0] + i, off[1] + j, off[2] + k, ivt) = 0.125 * s;
        }
      }
}

// a$D_restrict_tree (restrict:54-64): a$D_restrict_to_boxes on the parents
// of every level, from highest_lvl - 1 down to the coarsest
template <int D> void restrict_tree(Tree<D>& t, int iv, int ivt) {
  using T = Topo<D>;
  for (int lvl = t.highest_lvl - 1; lvl >= t.min_lvl; --lvl)
    for (int id : t.L(lvl).parents)
      for (int i_c = 0; i_c < T::NCH; ++i_c) {
        const int c_id = t.boxes[id].children[i_c];
        if (c_id == a5_no_box) continue;
        restrict_box_to<D>(t.boxes[c_id], t.boxes[id], iv, ivt);
      }
}

// a$D_gc_interp / a$D_gc_interp_lim (gc:155-358)
template <int D> void gc_interp(Tree<D>& t, int id, int nb, int iv, bool lim) {
  using T = Topo<D>;
  Box<D>& b = t.boxes[id];
  const int nc = b.n_cell;
  const int p_id = b.parent;
  Box<D>& pn = t.boxes[t.boxes[p_id].neighbors[nb - 1]];
  int off[D];
  child_offset(b, off);  // the tangential offsets (a$D_get_child_offset with nb differs in the normal one only)
  int ix, ix_f, ix_c;
  if (T::neighb_low(nb)) {
    ix = 0;
    ix_f = 1;
    ix_c = nc;
  } else {
    ix = nc + 1;
    ix_f = nc;
    ix_c = 1;
  }
  const double sixth = 1 / 6.0, third = 1 / 3.0;
  auto clip = [&](double& g, double c1) {
    if (lim && g > 2 * c1) g = 2 * c1;
  };
  if constexpr (D == 2) {
    for (int a = 1; a <= nc; ++a) {
      const int a_c1 = (T::neighb_dim(nb) == 0 ? off[1] : off[0]) + ((a + 1) >> 1);
      const int a_c2 = a_c1 + 1 - 2 * (a & 1);
      if (T::neighb_dim(nb) == 0) {
        const double c1 = pn.at(ix_c, a_c1, iv), c2 = pn.at(ix_c, a_c2, iv);
        double& g = b.at(ix, a, iv);
        g = 0.5 * c1 + sixth * c2 + third * b.at(ix_f, a, iv);
        clip(g, c1);
      } else {
        const double c1 = pn.at(a_c1, ix_c, iv), c2 = pn.at(a_c2, ix_c, iv);
        double& g = b.at(a, ix, iv);
        g = 0.5 * c1 + sixth * c2 + third * b.at(a, ix_f, iv);
        clip(g, c1);
      }
    }
  } else {
    for (int m = 1; m <= nc; ++m)
      for (int n = 1; n <= nc; ++n) {
        switch (T::neighb_dim(nb)) {
          case 0: {  // n = j, m = k
            const int j_c1 = off[1] + ((n + 1) >> 1), j_c2 = j_c1 + 1 - 2 * (n & 1);
            const int k_c1 = off[2] + ((m + 1) >> 1), k_c2 = k_c1 + 1 - 2 * (m & 1);
            const double c1 = pn.at(ix_c, j_c1, k_c1, iv), c2 = pn.at(ix_c, j_c2, k_c1, iv),
                         c3 = pn.at(ix_c, j_c1, k_c2, iv);
            double& g = b.at(ix, n, m, iv);
            g = third * c1 + sixth * c2 + sixth * c3 + third * b.at(ix_f, n, m, iv);
            clip(g, c1);
            break;
          }
          case 1: {  // n = i, m = k
            const int i_c1 = off[0] + ((n + 1) >> 1), i_c2 = i_c1 + 1 - 2 * (n & 1);
            const int k_c1 = off[2] + ((m + 1) >> 1), k_c2 = k_c1 + 1 - 2 * (m & 1);
            const double c1 = pn.at(i_c1, ix_c, k_c1, iv), c2 = pn.at(i_c2, ix_c, k_c1, iv),
                         c3 = pn.at(i_c1, ix_c, k_c2, iv);
            double& g = b.at(n, ix, m, iv);
            g = third * c1 + sixth * c2 + sixth * c3 + third * b.at(n, ix_f, m, iv);
            clip(g, c1);
            break;
          }
          default: {  // n = i, m = j
            const int i_c1 = off[0] + ((n + 1) >> 1), i_c2 = i_c1 + 1 - 2 * (n & 1);
            const int j_c1 = off[1] + ((m + 1) >> 1), j_c2 = j_c1 + 1 - 2 * (m & 1);
            const double c1 = pn.at(i_c1, j_c1, ix_c, iv), c2 = pn.at(i_c1, j_c2, ix_c, iv),
                         c3 = pn.at(i_c2, j_c1, ix_c, iv);
            double& g = b.at(n, m, ix, iv);
            g = third * c1 + sixth * c2 + sixth * c3 + third * b.at(n, m, ix_f, iv);
            clip(g, c1);
            break;
          }
        }
      }
  }
}

enum { RB_MG = 0, RB_PROLONG0 = 1, RB_INTERP = 2, RB_INTERP_LIM = 3 };
enum { BCM_TABLE = 0, BCM_DIRICHLET_ZERO = -1, BCM_NEUMANN_ZERO = -2 };

// a$D_gc_box (gc:50-69) for any variable, with the chosen sides_rb and sides_bc
template <int D> void gc_box_var(Tree<D>& t, int id, int iv, int rb, int bcm, const MG& mg) {
  using T = Topo<D>;
  for (int nb = 1; nb <= T::NNB; ++nb) {
    const int nb_id = t.boxes[id].neighbors[nb - 1];
    if (nb_id > a5_no_box) {
      sides_from_nb(t.boxes[id], t.boxes[nb_id], nb, iv);
    } else if (nb_id == a5_no_box) {
      switch (rb) {
        case RB_MG: sides_rb(t, id, nb, iv); break;
        case RB_PROLONG0: gc_prolong0(t, id, nb, iv); break;
        default: gc_interp(t, id, nb, iv, rb == RB_INTERP_LIM); break;
      }
    } else if (bcm == BCM_TABLE) {
      const int bc_type = sides_bc(t.boxes[id], id, nb, iv, mg);
      bc_to_gc(t.boxes[id], nb, iv, bc_type);
    } else {  // a$D_bc_dirichlet_zero / a$D_bc_neumann_zero, gc:361-378
      Box<D>& b = t.boxes[id];
      const int nc = b.n_cell, cmax = D == 3 ? nc : 1;
      for (int c = 1; c <= cmax; ++c)
        for (int a = 1; a <= nc; ++a) (&face_ghost<D>(b, nb, a, c))[(size_t)iv * b.nvol()] = 0.0;
      bc_to_gc(b, nb, iv, bcm == BCM_NEUMANN_ZERO ? a5_bc_neumann : a5_bc_dirichlet);
    }
  }
}

// a$D_gc_tree (gc:28-46)
template <int D> void gc_tree_var(Tree<D>& t, int iv, int rb, int bcm, const MG& mg) {
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl)
    for (int id : t.L(lvl).ids) gc_box_var<D>(t, id, iv, rb, bcm, mg);
}

// a$D_gc2_box (gc:420-440) with sides2_from_nb (:443-478), a$D_gc2_prolong1
// (:481-583) and a$D_bc2_neumann_zero (:586-632); gc_data is
// (nc[, nc], 2D), first index fastest
template <int D> void gc2_box(Tree<D>& t, int id, int iv, double* gc_data) {
  using T = Topo<D>;
  Box<D>& b = t.boxes[id];
  const int nc = b.n_cell;
  const int nf = D == 2 ? nc : nc * nc;
  for (int nb = 1; nb <= T::NNB; ++nb) {
    const int nb_id = b.neighbors[nb - 1];
    const int dim = T::neighb_dim(nb);
    double* side = gc_data + (size_t)(nb - 1) * nf;
    for (int m = 1; m <= (D == 3 ? nc : 1); ++m)
      for (int n = 1; n <= nc; ++n) {
        int c[3] = {0, 0, 0};
        {
          int tang[2] = {n, m}, e = 0;
          for (int d = 0; d < D; ++d)
            if (d != dim) c[d] = tang[e++];
        }
        double val;
        if (nb_id > a5_no_box) {
          c[dim] = T::neighb_low(nb) ? nc - 1 : 2;
          Box<D>& o = t.boxes[nb_id];
          val = D == 2 ? o.at(c[0], c[1], iv) : o.at(c[0], c[1], c[2], iv);
        } else if (nb_id == a5_no_box) {
          const int p_id = b.parent;
          Box<D>& pn = t.boxes[t.boxes[p_id].neighbors[nb - 1]];
          int off[D];
          child_offset(b, off);
          // a$D_get_child_offset(box, nb): minus neighb_dix * n_cell (lvl > 1)
          // or * n_cell/2 (sub-levels) in the normal direction
          off[dim] -= T::neighb_high_pm(nb) * (b.lvl > 1 ? nc : nc >> 1);
          const int ix = T::neighb_high_01(nb) * (nc + 3) - 1;
          int c1[3] = {0, 0, 0}, c2[3] = {0, 0, 0};
          for (int d = 0; d < D; ++d) {
            const int x = d == dim ? ix : c[d];
            c1[d] = off[d] + ((x + 1) >> 1);
            c2[d] = c1[d] + 1 - 2 * (x & 1);
          }
          if constexpr (D == 2)
            val = 0.5 * pn.at(c1[0], c1[1], iv) + 0.25 * pn.at(c2[0], c1[1], iv) + 0.25 * pn.at(c1[0], c2[1], iv);
          else
            val = 0.25 * pn.at(c1[0], c1[1], c1[2], iv) + 0.25 * pn.at(c2[0], c1[1], c1[2], iv) +
                  0.25 * pn.at(c1[0], c2[1], c1[2], iv) + 0.25 * pn.at(c1[0], c1[1], c2[2], iv);
        } else {
          c[dim] = T::neighb_low(nb) ? 2 : nc - 1;
          val = D == 2 ? b.at(c[0], c[1], iv) : b.at(c[0], c[1], c[2], iv);
        }
        side[(size_t)(n - 1) + (size_t)nc * (m - 1)] = val;
      }
  }
}

// flux_from_children (core:841-945, Cartesian): neighbour nb of box id has
// no children; its fluxes on the shared face become averages of the children's
template <int D> void flux_from_children(Tree<D>& t, int id, int nb, const std::vector<int>& f_ixs) {
  using T = Topo<D>;
  Box<D>& b = t.boxes[id];
  const int nc = b.n_cell, nch = nc >> 1;
  const int d = T::neighb_dim(nb);
  const int n_chnb = 1 << (D - 1);
  const int nb_id = b.neighbors[nb - 1];
  Box<D>& o = t.boxes[nb_id];
  const int i = T::neighb_low(nb) ? 1 : nc + 1, i_nb = T::neighb_low(nb) ? nc + 1 : 1;
  for (int ic = 0; ic < n_chnb; ++ic) {
    const int i_ch = T::child_adj_nb(ic, nb);
    Box<D>& c = t.boxes[b.children[i_ch - 1]];
    int ioff[D];
    for (int e = 0; e < D; ++e) ioff[e] = nch * T::child_dix(i_ch, e);
    for (int f : f_ixs) {
      if constexpr (D == 2) {
        for (int n = 1; n <= nch; ++n) {
          if (d == 0)
            o.f_at(f, 0, i_nb, ioff[1] + n, 1) = 0.5 * (c.f_at(f, 0, i, 2 * n - 1, 1) + c.f_at(f, 0, i, 2 * n, 1));
          else if (o.coord == 1) {  // cylindrical: weighted average (core:881-895)
            double w1, w2;
            cyl_child_weights(o.r_min[0], o.dr, ioff[0] + n, w1, w2);
            o.f_at(f, 1, ioff[0] + n, i_nb, 1) =
                0.5 * (w1 * c.f_at(f, 1, 2 * n - 1, i, 1) + w2 * c.f_at(f, 1, 2 * n, i, 1));
          } else {
            o.f_at(f, 1, ioff[0] + n, i_nb, 1) = 0.5 * (c.f_at(f, 1, 2 * n - 1, i, 1) + c.f_at(f, 1, 2 * n, i, 1));
          }
        }
      } else {
        for (int m = 1; m <= nch; ++m)
          for (int n = 1; n <= nch; ++n) {
            const int a = 2 * n - 1, bb = 2 * m - 1;
            switch (d) {
              case 0:
                o.f_at(f, 0, i_nb, ioff[1] + n, ioff[2] + m) =
                    0.25 * (c.f_at(f, 0, i, a, bb) + c.f_at(f, 0, i, a + 1, bb) + c.f_at(f, 0, i, a, bb + 1) +
                            c.f_at(f, 0, i, a + 1, bb + 1));
                break;
              case 1:
                o.f_at(f, 1, ioff[0] + n, i_nb, ioff[2] + m) =
                    0.25 * (c.f_at(f, 1, a, i, bb) + c.f_at(f, 1, a + 1, i, bb) + c.f_at(f, 1, a, i, bb + 1) +
                            c.f_at(f, 1, a + 1, i, bb + 1));
                break;
              default:
                o.f_at(f, 2, ioff[0] + n, ioff[1] + m, i_nb) =
                    0.25 * (c.f_at(f, 2, a, bb, i) + c.f_at(f, 2, a + 1, bb, i) + c.f_at(f, 2, a, bb + 1, i) +
                            c.f_at(f, 2, a + 1, bb + 1, i));
                break;
            }
          }
      }
    }
  }
}

// a$D_consistent_fluxes (core:811-838)
template <int D> void consistent_fluxes(Tree<D>& t, const std::vector<int>& f_ixs) {
  using T = Topo<D>;
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl - 1; ++lvl)
    for (int id : t.L(lvl).parents)
      for (int nb = 1; nb <= T::NNB; ++nb) {
        const int nb_id = t.boxes[id].neighbors[nb - 1];
        if (nb_id > a5_no_box && t.boxes[nb_id].children[0] == a5_no_box) flux_from_children<D>(t, id, nb, f_ixs);
      }
}

// a$D_write_vtk (io:115-310) with the m_vtk.f90 writer; the TIME and CYCLE
// field values are written as %.17E and %d text
template <int D>
int write_vtk(Tree<D>& t, const char* path, int n_cycle, double time, const std::vector<int>& icc,
              const std::vector<std::string>& cc_names, const std::vector<int>& ifc,
              const std::vector<std::string>& fc_names) {
  const int bc = t.n_cell, bn = t.n_cell + 1;
  const long long nodes_per_box = D == 2 ? bn * bn : bn * bn * bn;
  const long long cells_per_box = D == 2 ? bc * bc : bc * bc * bc;
  long long n_grids = 0;
  for (int lvl = 1; lvl <= t.highest_lvl; ++lvl) n_grids += (long long)t.L(lvl).leaves.size();
  const long long n_nodes = nodes_per_box * n_grids, n_cells = cells_per_box * n_grids;
  const int n_cc = (int)icc.size(), n_fc = (int)ifc.size(), ncol = n_cc + D * n_fc;
  std::vector<double> coords((size_t)(D * n_nodes));
  std::vector<double> cc_vars((size_t)(n_cells * ncol));  // column-major (cell, var)
  std::vector<int> offsets((size_t)n_cells), types((size_t)n_cells, D == 2 ? 8 : 11);
  std::vector<int> connects((size_t)((1 << D) * n_cells));
  long long ig = 0;
  const long long bn2 = (long long)bn * bn;
  for (int lvl = 1; lvl <= t.highest_lvl; ++lvl)
    for (int id : t.L(lvl).leaves) {
      Box<D>& b = t.boxes[id];
      ++ig;
      const long long cell_ix = (ig - 1) * cells_per_box, node_ix = (ig - 1) * nodes_per_box;
      for (int k = 1; k <= (D == 3 ? bn : 1); ++k)
        for (int j = 1; j <= bn; ++j)
          for (int i = 1; i <= bn; ++i) {
            const long long n_ix = D * (node_ix + (k - 1) * bn2 + (long long)(j - 1) * bn + i);
            const int ijk[3] = {i - 1, j - 1, k - 1};
            for (int d = 0; d < D; ++d) coords[(size_t)(n_ix - D + d)] = b.r_min[d] + ijk[d] * b.dr;
          }
      for (int k = 1; k <= (D == 3 ? bc : 1); ++k)
        for (int j = 1; j <= bc; ++j)
          for (int i = 1; i <= bc; ++i) {
            const long long n_ix = node_ix + (k - 1) * bn2 + (long long)(j - 1) * bn + i - 1;
            const long long c_ix = cell_ix + (long long)(k - 1) * bc * bc + (long long)(j - 1) * bc + i;
            for (int v = 0; v < n_cc; ++v)
              cc_vars[(size_t)(v * n_cells + c_ix - 1)] = D == 2 ? b.at(i, j, icc[v]) : b.at(i, j, k, icc[v]);
            for (int v = 0; v < n_fc; ++v)
              for (int d = 0; d < D; ++d) {
                double s = 0.0;
                s = s + b.f_at(ifc[v], d, i, j, k);
                s = s + b.f_at(ifc[v], d, i + (d == 0), j + (d == 1), k + (d == 2));
                cc_vars[(size_t)((n_cc + v * D + d) * n_cells + c_ix - 1)] = 0.5 * s;
              }
            offsets[(size_t)(c_ix - 1)] = (1 << D) * (int)c_ix;
            int* cn = &connects[(size_t)((1 << D) * (c_ix - 1))];
            cn[0] = (int)n_ix;
            cn[1] = (int)(n_ix + 1);
            cn[2] = (int)(n_ix + bn);
            cn[3] = (int)(n_ix + bn + 1);
            if (D == 3) {
              cn[4] = (int)(n_ix + bn2);
              cn[5] = (int)(n_ix + bn2 + 1);
              cn[6] = (int)(n_ix + bn2 + bn);
              cn[7] = (int)(n_ix + bn2 + bn + 1);
            }
          }
    }
  // m_vtk.f90: vtk_ini_xml .. vtk_end_xml
  std::string xml;
  std::vector<char> scratch;
  int indent = 0;
  long long offset = 0;
  auto w = [&](const std::string& s) { xml += std::string(indent, ' ') + s + "\n"; };
  auto dat = [&](const std::string& n, bool open) {
    if (open) {
      w("<" + n + ">");
      indent += 2;
    } else {
      indent -= 2;
      w("</" + n + ">");
    }
  };
  auto raw = [&](const void* p, long long n_bytes) {
    const int nb = (int)n_bytes;
    scratch.insert(scratch.end(), (const char*)&nb, (const char*)&nb + 4);
    scratch.insert(scratch.end(), (const char*)p, (const char*)p + n_bytes);
    offset += 4 + n_bytes;
  };
  xml = "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  indent = 2;
  dat("UnstructuredGrid", true);
  std::vector<float> wr((size_t)(3 * n_nodes), 0.0f);
  dat("FieldData", true);
  w("<DataArray type=\"Float64\" Name=\"TIME\" NumberOfTuples=\"1\" format=\"ascii\">");
  indent += 2;
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.17E", time);
  w(buf);
  dat("DataArray", false);
  w("<DataArray type=\"Int32\" Name=\"CYCLE\" NumberOfTuples=\"1\" format=\"ascii\">");
  indent += 2;
  w(std::to_string(n_cycle));
  dat("DataArray", false);
  dat("FieldData", false);
  for (int d = 0; d < D; ++d)
    for (long long n = 0; n < n_nodes; ++n) wr[(size_t)(3 * n + d)] = (float)coords[(size_t)(D * n + d)];
  w("<Piece NumberOfPoints=\"" + std::to_string(n_nodes) + "\" NumberOfCells=\"" + std::to_string(n_cells) + "\">");
  indent += 2;
  dat("Points", true);
  w("<DataArray type=\"Float32\" NumberOfComponents=\"3\" Name=\"Points\" format=\"appended\" offset=\"" +
    std::to_string(offset) + "\"/>");
  raw(wr.data(), 3 * n_nodes * 4);
  dat("Points", false);
  dat("Cells", true);
  w("<DataArray type=\"Int32\" Name=\"connectivity\" format=\"appended\" offset=\"" + std::to_string(offset) + "\"/>");
  raw(connects.data(), (n_cells ? (long long)offsets[(size_t)(n_cells - 1)] : 0) * 4);
  w("<DataArray type=\"Int32\" Name=\"offsets\" format=\"appended\" offset=\"" + std::to_string(offset) + "\"/>");
  raw(offsets.data(), n_cells * 4);
  w("<DataArray type=\"Int32\" Name=\"types\" format=\"appended\" offset=\"" + std::to_string(offset) + "\"/>");
  raw(types.data(), n_cells * 4);
  dat("Cells", false);
  dat("CellData", true);
  std::vector<std::string> names(cc_names);
  const bool cyl = D == 2 && t.coord == 1;  // io:174-176
  const char* sfx[3] = {cyl ? "_r" : "_x", cyl ? "_z" : "_y", "_z"};
  for (int v = 0; v < n_fc; ++v)
    for (int d = 0; d < D; ++d) names.push_back(fc_names[(size_t)v] + sfx[d]);
  for (int c = 0; c < ncol; ++c) {
    w("<DataArray type=\"Float64\" Name=\"" + names[(size_t)c] +
      "\" NumberOfComponents=\"1\" format=\"appended\" offset=\"" + std::to_string(offset) + "\"/>");
    raw(cc_vars.data() + (size_t)c * n_cells, n_cells * 8);
  }
  dat("CellData", false);
  dat("Piece", false);  // vtk_unstr_geo_xml_close
  dat("UnstructuredGrid", false);
  w("<AppendedData encoding=\"raw\">");
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return -1;
  std::fwrite(xml.data(), 1, xml.size(), fp);
  std::fputc('_', fp);
  if (!scratch.empty()) std::fwrite(scratch.data(), 1, scratch.size(), fp);
  std::string tail = "\n" + std::string(indent, ' ') + "</AppendedData>\n";
  indent -= 2;
  tail += std::string(indent, ' ') + "</VTKFile>\n";
  std::fwrite(tail.data(), 1, tail.size(), fp);
  std::fclose(fp);
  return 0;
}

struct OrcHandle {
  int dim;
  void* tree;
  MG mg;
};

template <int D> static Tree<D>& TT(OrcHandle* h) { return *static_cast<Tree<D>*>(h->tree); }

#define DISPATCH(h, expr2, expr3) ((h)->dim == 2 ? (expr2) : (expr3))

extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// a$D_init + a$D_set_base. n_var = 3 (phi, rhs, tmp).
OrcHandle* orc_tree_new(int dim, int n_cell, double dr, const double* r_min, int lvl_limit,
                        int coarsen_to, int n_base, const int* ix_list, const int* nb_list_in) {
  if (dim != 2 && dim != 3) return nullptr;
  std::vector<int> nb_list(nb_list_in, nb_list_in + (size_t)n_base * 2 * dim);
  auto* h = new OrcHandle();
  h->dim = dim;
  if (dim == 2) {
    Tree<2>* t = tree_init<2>(n_cell, 3, dr, r_min, lvl_limit, 1000, coarsen_to, 256.0);
    if (!t || set_base<2>(*t, n_base, ix_list, nb_list.data()) != 0) {
      delete t;
      delete h;
      return nullptr;
    }
    h->tree = t;
  } else {
    Tree<3>* t = tree_init<3>(n_cell, 3, dr, r_min, lvl_limit, 1000, coarsen_to, 256.0);
    if (!t || set_base<3>(*t, n_base, ix_list, nb_list.data()) != 0) {
      delete t;
      delete h;
      return nullptr;
    }
    h->tree = t;
  }
  return h;
}

void orc_tree_free(OrcHandle* h) {
  if (!h) return;
  if (h->dim == 2)
    delete static_cast<Tree<2>*>(h->tree);
  else
    delete static_cast<Tree<3>*>(h->tree);
  delete h;
}

static RefCrit make_crit(int dim, int kind, int lvl_max, double thr, double prob, uint64_t seed,
                         int src_lpl, int n_gauss, const double* gauss) {
  RefCrit rc;
  rc.src_lpl = src_lpl;
  rc.kind = kind;
  rc.lvl_max = lvl_max;
  rc.thr = thr;
  rc.prob = prob;
  rc.seed = seed;
  if (n_gauss > 0) rc.gauss.assign(gauss, gauss + (size_t)n_gauss * (2 + dim));
  return rc;
}

// One call of a$D_adjust_refinement with a built-in refinement criterion.
int orc_adjust_refinement(OrcHandle* h, int kind, int lvl_max, double thr, double prob,
                          unsigned long long seed, int src_lpl, int n_gauss, const double* gauss,
                          int* n_add, int* n_rm) {
  RefCrit rc = make_crit(h->dim, kind, lvl_max, thr, prob, seed, src_lpl, n_gauss, gauss);
  return DISPATCH(h, adjust_refinement<2>(TT<2>(h), rc, n_add, n_rm),
                  adjust_refinement<3>(TT<3>(h), rc, n_add, n_rm));
}

int orc_min_lvl(OrcHandle* h) { return DISPATCH(h, TT<2>(h).min_lvl, TT<3>(h).min_lvl); }
int orc_highest_lvl(OrcHandle* h) { return DISPATCH(h, TT<2>(h).highest_lvl, TT<3>(h).highest_lvl); }
int orc_highest_id(OrcHandle* h) { return DISPATCH(h, TT<2>(h).highest_id, TT<3>(h).highest_id); }

}  // extern "C"
template <int D>
static void export_boxes(Tree<D>& t, int* lvl, int* ix, int* parent, int* children, int* neighbors,
                         int* n_cell, double* dr, double* r_min, int* in_use) {
  constexpr int NCH = 1 << D, NNB = 2 * D;
  for (int id = 1; id <= t.highest_id; ++id) {
    Box<D>& b = t.boxes[id];
    int k = id - 1;
    lvl[k] = b.lvl;
    parent[k] = b.parent;
    n_cell[k] = b.n_cell;
    dr[k] = b.dr;
    in_use[k] = b.in_use ? 1 : 0;
    for (int d = 0; d < D; ++d) {
      ix[k * D + d] = b.ix[d];
      r_min[k * D + d] = b.r_min[d];
    }
    for (int c = 0; c < NCH; ++c) children[k * NCH + c] = b.children[c];
    for (int nb = 0; nb < NNB; ++nb) neighbors[k * NNB + nb] = b.neighbors[nb];
  }
}
extern "C" {

// Per-id topology (arrays sized by highest_id, id-1 indexed).
void orc_export_boxes(OrcHandle* h, int* lvl, int* ix, int* parent, int* children, int* neighbors,
                      int* n_cell, double* dr, double* r_min, int* in_use) {
  if (h->dim == 2)
    export_boxes<2>(TT<2>(h), lvl, ix, parent, children, neighbors, n_cell, dr, r_min, in_use);
  else
    export_boxes<3>(TT<3>(h), lvl, ix, parent, children, neighbors, n_cell, dr, r_min, in_use);
}

}  // extern "C"
template <int D> static void level_sizes(Tree<D>& t, int lvl, int* out) {
  Lvl& L = t.L(lvl);
  out[0] = (int)L.ids.size();
  out[1] = (int)L.leaves.size();
  out[2] = (int)L.parents.size();
}
extern "C" {
void orc_level_sizes(OrcHandle* h, int lvl, int* out3) {
  if (h->dim == 2)
    level_sizes<2>(TT<2>(h), lvl, out3);
  else
    level_sizes<3>(TT<3>(h), lvl, out3);
}

}  // extern "C"
template <int D> static void level_lists(Tree<D>& t, int lvl, int* ids, int* leaves, int* parents) {
  Lvl& L = t.L(lvl);
  std::copy(L.ids.begin(), L.ids.end(), ids);
  std::copy(L.leaves.begin(), L.leaves.end(), leaves);
  std::copy(L.parents.begin(), L.parents.end(), parents);
}
extern "C" {
void orc_level_lists(OrcHandle* h, int lvl, int* ids, int* leaves, int* parents) {
  if (h->dim == 2)
    level_lists<2>(TT<2>(h), lvl, ids, leaves, parents);
  else
    level_lists<3>(TT<3>(h), lvl, ids, leaves, parents);
}

// Variable iv of all boxes of one level, in the level's id order, each box as
// its full (n_cell+2)^D array.
}  // extern "C"
template <int D> static void level_cc(Tree<D>& t, int lvl, int iv, double* buf, bool get) {
  size_t off = 0;
  for (int id : t.L(lvl).ids) {
    Box<D>& b = t.boxes[id];
    double* v = b.var(iv);
    if (get)
      std::copy(v, v + b.nvol(), buf + off);
    else
      std::copy(buf + off, buf + off + b.nvol(), v);
    off += b.nvol();
  }
}
extern "C" {
void orc_get_level_cc(OrcHandle* h, int lvl, int iv, double* out) {
  if (h->dim == 2)
    level_cc<2>(TT<2>(h), lvl, iv, out, true);
  else
    level_cc<3>(TT<3>(h), lvl, iv, out, true);
}
void orc_set_level_cc(OrcHandle* h, int lvl, int iv, double* in) {
  if (h->dim == 2)
    level_cc<2>(TT<2>(h), lvl, iv, in, false);
  else
    level_cc<3>(TT<3>(h), lvl, iv, in, false);
}

// cc(..., iv) := 0 on every box of every level, ghosts included
// (a$D_box_clear_cc, src/m_aX_utils.f90:262-270, on all boxes).
void orc_zero_var(OrcHandle* h, int iv);

// rhs (or any iv) := sum of Gaussians at the cell centres of every box.
}  // extern "C"
template <int D> static void zero_var(Tree<D>& t, int iv) {
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl) {
    const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp parallel for
    for (int n = 0; n < (int)ids.size(); ++n) {
      Box<D>& b = t.boxes[ids[n]];
      std::fill(b.cc.begin() + (size_t)iv * b.nvol(), b.cc.begin() + (size_t)(iv + 1) * b.nvol(), 0.0);
    }
  }
}
extern "C" void orc_zero_var(OrcHandle* h, int iv) {
  if (h->dim == 2)
    zero_var<2>(TT<2>(h), iv);
  else
    zero_var<3>(TT<3>(h), iv);
}
template <int D> static void fill_gauss(Tree<D>& t, int iv, int lpl, const std::vector<double>& g) {
  for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl) {
    const std::vector<int>& ids = t.L(lvl).ids;
#pragma omp parallel for
    for (int n = 0; n < (int)ids.size(); ++n) {
      Box<D>& b = t.boxes[ids[n]];
      int nc = b.n_cell;
      int kmax = (D == 3) ? nc : 1;
      for (int k = 1; k <= kmax; ++k)
        for (int j = 1; j <= nc; ++j)
          for (int i = 1; i <= nc; ++i) {
            int cix[3] = {i, j, k};
            double r[3];
            r_cc<D>(b, cix, r);
            double f = source_at<D>(g, lpl, r);
            if constexpr (D == 2)
              b.at(i, j, iv) = f;
            else
              b.at(i, j, k, iv) = f;
          }
    }
  }
}
extern "C" {
void orc_fill_gauss(OrcHandle* h, int iv, int lpl, int n_gauss, const double* gauss) {
  std::vector<double> g(gauss, gauss + (size_t)n_gauss * (2 + h->dim));
  if (h->dim == 2)
    fill_gauss<2>(TT<2>(h), iv, lpl, g);
  else
    fill_gauss<3>(TT<3>(h), iv, lpl, g);
}

// mg$D_init_mg with the defaults of mg:142-151 for negative cycle counts.
void orc_mg_init(OrcHandle* h, int n_down, int n_up, int n_base, int bc_kind, int n_gauss,
                 const double* gauss) {
  MG& mg = h->mg;
  mg.n_cycle_down = n_down < 0 ? 2 : n_down;
  mg.n_cycle_up = n_up < 0 ? 2 : n_up;
  mg.n_cycle_base = n_base < 0 ? 2 : n_base;
  mg.bc_kind = bc_kind;
  mg.bc_gauss.assign(gauss ? gauss : nullptr, gauss ? gauss + (size_t)n_gauss * (2 + h->dim) : nullptr);
  mg.initialized = true;
}

// Per-face boundary records for BC_TABLE: face i is (ids[i], faces[i]
// 0-based), its type types[i] (a5_bc_dirichlet / a5_bc_neumann) and nc^(D-1)
// values of that box's n_cell, consecutive in face order.
void orc_mg_set_bc_table(OrcHandle* h, int n_faces, const int* ids, const int* faces,
                         const int* types, const double* values) {
  MG& mg = h->mg;
  int D = h->dim, NNB = 2 * D;
  int hid = D == 2 ? TT<2>(h).highest_id : TT<3>(h).highest_id;
  mg.tab_type.assign((size_t)(hid + 1) * NNB, a5_bc_dirichlet);
  mg.tab_off.assign((size_t)(hid + 1) * NNB, -1);
  mg.tab_vals.clear();
  for (int i = 0; i < n_faces; ++i) {
    int nc = D == 2 ? TT<2>(h).boxes[ids[i]].n_cell : TT<3>(h).boxes[ids[i]].n_cell;
    size_t k = (size_t)ids[i] * NNB + faces[i];
    mg.tab_type[k] = types[i];
    mg.tab_off[k] = (long long)mg.tab_vals.size();
    long long nfc = D == 2 ? nc : (long long)nc * nc;
    mg.tab_vals.insert(mg.tab_vals.end(), values, values + nfc);
    values += nfc;
  }
  mg.bc_kind = BC_TABLE;
}

void orc_vcycle(OrcHandle* h, int highest_lvl, int set_residual) {
  if (h->dim == 2)
    fas_vcycle<2>(TT<2>(h), h->mg, highest_lvl, set_residual != 0);
  else
    fas_vcycle<3>(TT<3>(h), h->mg, highest_lvl, set_residual != 0);
}

void orc_fmg(OrcHandle* h, int set_residual, int have_guess) {
  if (h->dim == 2)
    fas_fmg<2>(TT<2>(h), h->mg, set_residual != 0, have_guess != 0);
  else
    fas_fmg<3>(TT<3>(h), h->mg, set_residual != 0, have_guess != 0);
}

// Per-operator entry points for fine-grained parity tests.
void orc_gsrb_level(OrcHandle* h, int lvl, int n_cycle) {
  if (h->dim == 2)
    gsrb_boxes<2>(TT<2>(h), TT<2>(h).L(lvl).ids, h->mg, n_cycle);
  else
    gsrb_boxes<3>(TT<3>(h), TT<3>(h).L(lvl).ids, h->mg, n_cycle);
}
void orc_fill_gc_level(OrcHandle* h, int lvl) {
  if (h->dim == 2)
    fill_gc_phi<2>(TT<2>(h), TT<2>(h).L(lvl).ids, h->mg);
  else
    fill_gc_phi<3>(TT<3>(h), TT<3>(h).L(lvl).ids, h->mg);
}
void orc_update_coarse(OrcHandle* h, int lvl) {
  if (h->dim == 2)
    update_coarse<2>(TT<2>(h), lvl, h->mg);
  else
    update_coarse<3>(TT<3>(h), lvl, h->mg);
}
void orc_correct_children(OrcHandle* h, int lvl_parent) {
  if (h->dim == 2)
    correct_children<2>(TT<2>(h), TT<2>(h).L(lvl_parent).parents, h->mg);
  else
    correct_children<3>(TT<3>(h), TT<3>(h).L(lvl_parent).parents, h->mg);
}
void orc_gc_tree(OrcHandle* h) {  // a$D_gc_tree for i_phi, gc:28-46
  if (h->dim == 2) {
    Tree<2>& t = TT<2>(h);
    for (int l = t.min_lvl; l <= t.highest_lvl; ++l) fill_gc_phi<2>(t, t.L(l).ids, h->mg);
  } else {
    Tree<3>& t = TT<3>(h);
    for (int l = t.min_lvl; l <= t.highest_lvl; ++l) fill_gc_phi<3>(t, t.L(l).ids, h->mg);
  }
}
// Residual tmp = rhs - L(phi) on every box of every level (the set_residual
// branch of mg:243-254).
void orc_residual_all(OrcHandle* h) {
  if (h->dim == 2) {
    Tree<2>& t = TT<2>(h);
    for (int l = t.min_lvl; l <= t.highest_lvl; ++l)
      for (int id : t.L(l).ids) residual_box<2>(t.boxes[id], h->mg);
  } else {
    Tree<3>& t = TT<3>(h);
    for (int l = t.min_lvl; l <= t.highest_lvl; ++l)
      for (int id : t.L(l).ids) residual_box<3>(t.boxes[id], h->mg);
  }
}

double orc_tree_max_cc(OrcHandle* h, int iv) {
  return DISPATCH(h, tree_max_cc<2>(TT<2>(h), iv, true), tree_max_cc<3>(TT<3>(h), iv, true));
}
double orc_tree_min_cc(OrcHandle* h, int iv) {
  return DISPATCH(h, tree_max_cc<2>(TT<2>(h), iv, false), tree_max_cc<3>(TT<3>(h), iv, false));
}
double orc_leaf_mean(OrcHandle* h, int iv) {
  return DISPATCH(h, leaf_mean<2>(TT<2>(h), iv), leaf_mean<3>(TT<3>(h), iv));
}

// Morton helpers for the known-answer test of tests/test_morton.f90.
unsigned long long orc_morton_from_ix(int dim, const int* ix) {
  return dim == 2 ? morton_from_ix<2>(ix) : morton_from_ix<3>(ix);
}
void orc_morton_to_ix(int dim, unsigned long long m, int* ix) {
  if (dim == 2) {
    ix[0] = bit_despace_1(m);
    ix[1] = bit_despace_1(m >> 1);
  } else {
    ix[0] = bit_despace_2(m);
    ix[1] = bit_despace_2(m >> 1);
    ix[2] = bit_despace_2(m >> 2);
  }
}

// Topology table accessors (1-based in, 1-based out).
int orc_child_rev(int dim, int c, int d) {
  return dim == 2 ? Topo<2>::child_rev(c, d - 1) : Topo<3>::child_rev(c, d - 1);
}
int orc_child_adj_nb(int dim, int k, int nb) {
  return dim == 2 ? Topo<2>::child_adj_nb(k - 1, nb) : Topo<3>::child_adj_nb(k - 1, nb);
}
int orc_child_dix(int dim, int d, int c) {
  return dim == 2 ? Topo<2>::child_dix(c, d - 1) : Topo<3>::child_dix(c, d - 1);
}
int orc_neighb_rev(int dim, int nb) {
  return dim == 2 ? Topo<2>::neighb_rev(nb) : Topo<3>::neighb_rev(nb);
}
int orc_neighb_dix(int dim, int d, int nb) {
  return dim == 2 ? Topo<2>::neighb_dix(nb, d - 1) : Topo<3>::neighb_dix(nb, d - 1);
}
int orc_ix_to_ichild(int dim, const int* ix) {
  return dim == 2 ? Topo<2>::ix_to_ichild(ix) : Topo<3>::ix_to_ichild(ix);
}


// General ghost-cell, transfer and output routines (see above).
void orc_add_vars(OrcHandle* h, int n_cc, int n_fc) {
  if (h->dim == 2)
    add_vars<2>(TT<2>(h), n_cc, n_fc);
  else
    add_vars<3>(TT<3>(h), n_cc, n_fc);
}
static long long fc_io(OrcHandle* h, int ifc, double* buf, bool get) {
  long long off = 0;
  auto go = [&](auto& t) {
    for (int lvl = t.min_lvl; lvl <= t.highest_lvl; ++lvl)
      for (int id : t.L(lvl).ids) {
        auto& b = t.boxes[id];
        const long long n = (long long)(h->dim) * b.fblock();
        double* v = b.fc.data() + (size_t)ifc * n;
        if (buf) {
          if (get)
            std::copy(v, v + n, buf + off);
          else
            std::copy(buf + off, buf + off + n, v);
        }
        off += n;
      }
  };
  if (h->dim == 2)
    go(TT<2>(h));
  else
    go(TT<3>(h));
  return off;
}
long long orc_fc_count(OrcHandle* h) { return fc_io(h, 0, nullptr, true); }
void orc_get_fc(OrcHandle* h, int ifc, double* out) { fc_io(h, ifc, out, true); }
void orc_set_fc(OrcHandle* h, int ifc, double* in) { fc_io(h, ifc, in, false); }
void orc_prolong_from_level(OrcHandle* h, int lvl, int iv, int iv_to, int order, int add) {
  if (h->dim == 2)
    prolong_from_level<2>(TT<2>(h), lvl, iv, iv_to, order, add != 0);
  else
    prolong_from_level<3>(TT<3>(h), lvl, iv, iv_to, order, add != 0);
}
void orc_restrict_tree(OrcHandle* h, int iv, int iv_to) {
  if (h->dim == 2)
    restrict_tree<2>(TT<2>(h), iv, iv_to);
  else
    restrict_tree<3>(TT<3>(h), iv, iv_to);
}
void orc_gc_tree_var(OrcHandle* h, int iv, int rb, int bcm) {
  if (h->dim == 2)
    gc_tree_var<2>(TT<2>(h), iv, rb, bcm, h->mg);
  else
    gc_tree_var<3>(TT<3>(h), iv, rb, bcm, h->mg);
}
// a$D_gc2_box on every box of a level (level-list order), (nc[,nc], 2D) each
void orc_gc2_level(OrcHandle* h, int lvl, int iv, double* out) {
  auto go = [&](auto& t, int D) {
    const int nc = t.n_cell;
    const long long per = 2LL * D * (D == 2 ? nc : nc * nc);
    long long off = 0;
    for (int id : t.L(lvl).ids) {
      if (D == 2)
        gc2_box<2>(TT<2>(h), id, iv, out + off);
      else
        gc2_box<3>(TT<3>(h), id, iv, out + off);
      off += per;
    }
  };
  if (h->dim == 2)
    go(TT<2>(h), 2);
  else
    go(TT<3>(h), 3);
}
void orc_consistent_fluxes(OrcHandle* h, int n, const int* f_ixs) {
  std::vector<int> f(f_ixs, f_ixs + n);
  if (h->dim == 2)
    consistent_fluxes<2>(TT<2>(h), f);
  else
    consistent_fluxes<3>(TT<3>(h), f);
}
int orc_write_vtk(OrcHandle* h, const char* path, int n_cycle, double time, int n_cc, const int* icc,
                  const char* const* cc_names, int n_fc, const int* ifc, const char* const* fc_names) {
  std::vector<int> a(icc, icc + n_cc), b(ifc, ifc + n_fc);
  std::vector<std::string> an(cc_names, cc_names + n_cc), bn(fc_names, fc_names + n_fc);
  return h->dim == 2 ? write_vtk<2>(TT<2>(h), path, n_cycle, time, a, an, b, bn)
                     : write_vtk<3>(TT<3>(h), path, n_cycle, time, a, an, b, bn);
}


// mg%box_op / box_gsrb / box_corr / box_rstr with mg%i_eps, mg%i_lsf and
// mg%i_bval; box tags are taken again at their next use (the reference's
// a5_init_tag state). Returns -1 when a box would take two tags (where
// mg$D_set_box_tag stops).
int orc_mg_set_operator(OrcHandle* h, int op, int i_eps, int i_lsf, int i_bval) {
  h->mg.op = op;
  h->mg.i_eps = i_eps;
  h->mg.i_lsf = i_lsf;
  h->mg.i_bval = i_bval;
  int ok = 1;
  auto reset = [&](auto& t) {
    for (size_t id = 1; id < t.boxes.size(); ++id) {
      t.boxes[id].tag = a5_init_tag;
      if (op == OP_AUTO && t.boxes[id].in_use && !set_box_tag(t.boxes[id], h->mg)) ok = 0;
      t.boxes[id].tag = a5_init_tag;
    }
  };
  if (h->dim == 2)
    reset(TT<2>(h));
  else
    reset(TT<3>(h));
  return ok ? 0 : -1;
}

// a$D_init's coord argument (core:58-70, 102, 198): a5_cyl for a 2-D tree,
// set on the tree and its boxes.
int orc_set_coord(OrcHandle* h, int coord) {
  if (h->dim != 2 && coord == 1) return -1;
  auto& t = TT<2>(h);
  t.coord = coord;
  for (size_t id = 1; id < t.boxes.size(); ++id) t.boxes[id].coord = coord;
  return 0;
}

}  // extern "C"
