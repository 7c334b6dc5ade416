// Host tree build. Restates src/m_aX_core.f90:24-787 and src/m_morton.f90 so
// that box ids, levels, neighbour and child links come out identical to the
// reference's; the device planner then reorders boxes by Morton key.
#include "host_tree.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace afv {

namespace {

// Interleave the bits of x with one (dim 2) or two (dim 3) zero bits,
// src/m_morton.f90:96-136. The 3-D form keeps 21 bits of each index.
uint64_t spread2(uint32_t v) {
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
uint64_t spread3(uint32_t v) {
  uint64_t x = v & 0x1fffffu;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

// Tables of src/m_aX_t.f90:54-149 expressed through the child number bits.
inline int nb_dim(int nb1) { return (nb1 - 1) >> 1; }          // nb1: 1-based
inline int nb_high(int nb1) { return (nb1 - 1) & 1; }          // a$D_neighb_high_01
inline int nb_rev(int nb1) { return nb_high(nb1) ? nb1 - 1 : nb1 + 1; }

uint64_t mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

}  // namespace

uint64_t morton_key(int dim, const int* ix0) {
  if (dim == 2) return spread2((uint32_t)ix0[0]) | (spread2((uint32_t)ix0[1]) << 1);
  return spread3((uint32_t)ix0[0]) | (spread3((uint32_t)ix0[1]) << 1) |
         (spread3((uint32_t)ix0[2]) << 2);
}

int HostTree::n_used() const {
  int n = 0;
  for (int l = min_lvl; l <= highest_lvl; ++l) n += (int)L(l).ids.size();
  return n;
}

// a$D_ix_to_ichild, src/m_aX_t.f90:378-387
int HostTree::ichild_of(int id) const {
  int c = nch;
  for (int d = 0; d < dim; ++d) c -= (ix[(size_t)id * dim + d] & 1) << d;
  return c;
}

void HostTree::resize(int new_size) {
  size_t n = (size_t)new_size + 1;
  lvl.resize(n, 0);
  parent.resize(n, 0);
  ncell.resize(n, 0);
  in_use.resize(n, 0);
  ix.resize(n * dim, 0);
  children.resize(n * nch, 0);
  neighbors.resize(n * nnb, 0);
  dr.resize(n, 0.0);
  r_min.resize(n * dim, 0.0);
}

void HostTree::get_free_ids(int n, int* out) {  // core:609-621
  for (int i = 0; i < n; ++i) out[i] = highest_id + 1 + i;
  highest_id += n;
}

void HostTree::lists_of(LevelLists& lv) {  // set_leaves_parents, core:317-348
  lv.leaves.clear();
  lv.parents.clear();
  for (int id : lv.ids) (has_children(id) ? lv.parents : lv.leaves).push_back(id);
}

int HostTree::init(int dim_, int n_cell_, double dr_, const double* rmin, int lvl_limit_,
                   int coarsen_to, double mem_limit_gb, std::string& err) {
  if (dim_ != 2 && dim_ != 3) return err = "dim must be 2 or 3", AFV_ERR_INVALID;
  if (n_cell_ < 2) return err = "n_cell should be >= 2", AFV_ERR_INVALID;
  if (n_cell_ & 1) return err = "n_cell should be even", AFV_ERR_INVALID;
  if (lvl_limit_ <= 0) return err = "lvl_limit should be > 0", AFV_ERR_INVALID;
  if (!(mem_limit_gb > 0)) return err = "mem_limit_gb should be > 0", AFV_ERR_INVALID;
  if (!(dr_ > 0)) return err = "dr should be > 0", AFV_ERR_INVALID;
  dim = dim_;
  nch = 1 << dim;
  nnb = 2 * dim;
  n_cell = n_cell_;
  lvl_limit = lvl_limit_;
  dr_base = dr_;
  for (int d = 0; d < 3; ++d) r_base[d] = (rmin && d < dim) ? rmin[d] : 0.0;
  min_lvl = 1;
  if (coarsen_to > 0) {  // core:74-83
    min_lvl = 1 - (int)std::lround(std::log((double)n_cell / coarsen_to) / std::log(2.0));
    if (min_lvl > 1 || (1 << (1 - min_lvl)) * coarsen_to != n_cell)
      return err = "cannot coarsen to given value", AFV_ERR_INVALID;
  }
  levels.assign((size_t)(lvl_limit + 2 - min_lvl), LevelLists());
  resize(1000);
  highest_id = 0;
  highest_lvl = 0;
  // Box size of a$D_box_bytes (src/m_aX_t.f90:331-341) for phi, rhs, tmp,
  // with a fixed overhead in place of the compiler's storage_size of box$D_t.
  double vol = std::pow((double)(n_cell + 2), dim);
  double box_bytes = 8.0 * 3 * vol + 256.0;
  box_limit = (int)std::min(2.0e9, std::round(mem_limit_gb * 1073741824.0 / box_bytes));
  return AFV_OK;
}

int HostTree::set_base(int n_boxes, const int* ix_list, int* nb_list, std::string& err) {
  if (levels.empty()) return err = "tree not initialised", AFV_ERR_STATE;
  if (highest_id > 0) return err = "this tree already has boxes", AFV_ERR_STATE;
  if (n_boxes <= 0) return err = "need at least one base box", AFV_ERR_INVALID;
  for (int i = 0; i < n_boxes * dim; ++i)
    if (ix_list[i] < 1) return err = "need all ix_list > 0", AFV_ERR_INVALID;
  for (int i = 0; i < n_boxes * nnb; ++i)
    if (nb_list[i] > n_boxes) return err = "neighbour id out of range", AFV_ERR_INVALID;
  // Neighbours only given from one side are mirrored (core:163-172).
  for (int i = 1; i <= n_boxes; ++i)
    for (int nb = 1; nb <= nnb; ++nb) {
      int v = nb_list[(i - 1) * nnb + nb - 1];
      if (v > kNoBox && v != i) nb_list[(v - 1) * nnb + nb_rev(nb) - 1] = i;
    }
  for (int i = 0; i < n_boxes * nnb; ++i)
    if (nb_list[i] == kNoBox) return err = "unresolved neighbors", AFV_ERR_INVALID;
  if (n_boxes > capacity()) resize(n_boxes);

  // Levels min_lvl..1 are copies of the base with n_cell halved per level down.
  for (int l = min_lvl; l <= 1; ++l) {
    LevelLists& lv = L(l);
    lv.ids.assign(n_boxes, 0);
    get_free_ids(n_boxes, lv.ids.data());
    int offset = lv.ids[0] - 1;
    for (int i = 0; i < n_boxes; ++i) {
      int id = lv.ids[i];
      lvl[id] = l;
      for (int d = 0; d < dim; ++d) {
        ix[(size_t)id * dim + d] = ix_list[i * dim + d];
        r_min[(size_t)id * dim + d] = r_base[d] + (ix_list[i * dim + d] - 1) * dr_base * n_cell;
      }
      dr[id] = dr_base * std::pow(0.5, l - 1);
      ncell[id] = n_cell / (1 << (1 - l));
      parent[id] = kNoBox;
      std::fill_n(&children[(size_t)id * nch], nch, kNoBox);
      for (int nb = 0; nb < nnb; ++nb) {
        int v = nb_list[i * nnb + nb];
        neighbors[(size_t)id * nnb + nb] = v > kNoBox ? v + offset : v;
      }
      in_use[id] = 1;
    }
    if (l == 1)
      lv.leaves = lv.ids;
    else
      lv.parents = lv.ids;
    if (l > min_lvl) {
      const LevelLists& below = L(l - 1);
      for (int i = 0; i < n_boxes; ++i) {
        children[(size_t)below.ids[i] * nch] = lv.ids[i];
        parent[lv.ids[i]] = below.ids[i];
      }
    }
  }
  highest_lvl = 1;
  ready = true;
  return AFV_OK;
}

// a$D_tidy_up, core:238-314: when more than max_hole_frac of the ids are holes
// (and at least n_clean_min can be reclaimed), renumber boxes level by level in
// Morton order.
void HostTree::tidy_up(double max_hole_frac, int n_clean_min) {
  int used = n_used();
  double hole_frac = 1 - used / (double)highest_id;
  int n_clean = (int)std::lround(hole_frac * highest_id);
  if (!(hole_frac > max_hole_frac && n_clean >= n_clean_min)) return;

  std::vector<int> map((size_t)highest_id + 1, 0), order;
  order.reserve(used);
  for (int l = min_lvl; l <= highest_lvl; ++l) {
    LevelLists& lv = L(l);
    std::vector<uint64_t> key(lv.ids.size());
    for (size_t n = 0; n < lv.ids.size(); ++n) {
      int ix0[3];
      for (int d = 0; d < dim; ++d) ix0[d] = ix[(size_t)lv.ids[n] * dim + d] - 1;
      key[n] = morton_key(dim, ix0);
    }
    std::vector<int> perm(lv.ids.size());
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<int> sorted(lv.ids.size());
    for (size_t n = 0; n < perm.size(); ++n) sorted[n] = lv.ids[perm[n]];
    for (int old_id : sorted) {
      order.push_back(old_id);
      map[old_id] = (int)order.size();
    }
    for (size_t n = 0; n < sorted.size(); ++n) lv.ids[n] = map[sorted[n]];
  }
  // Gather into the new numbering, then translate the links.
  HostTree old = *this;
  for (int nid = 1; nid <= used; ++nid) {
    int o = order[nid - 1];
    lvl[nid] = old.lvl[o];
    ncell[nid] = old.ncell[o];
    in_use[nid] = 1;
    dr[nid] = old.dr[o];
    parent[nid] = map[old.parent[o]];
    for (int d = 0; d < dim; ++d) {
      ix[(size_t)nid * dim + d] = old.ix[(size_t)o * dim + d];
      r_min[(size_t)nid * dim + d] = old.r_min[(size_t)o * dim + d];
    }
    for (int c = 0; c < nch; ++c) children[(size_t)nid * nch + c] = map[old.children[(size_t)o * nch + c]];
    for (int nb = 0; nb < nnb; ++nb) {
      int v = old.neighbors[(size_t)o * nnb + nb];
      neighbors[(size_t)nid * nnb + nb] = v > kNoBox ? map[v] : v;
    }
  }
  for (int id = used + 1; id <= highest_id; ++id) in_use[id] = 0;
  for (int l = min_lvl; l <= highest_lvl; ++l) lists_of(L(l));
  highest_id = used;
}

void HostTree::make_view(int id, afv_box_view* v) const {
  v->id = id;
  v->lvl = lvl[id];
  v->n_cell = ncell[id];
  v->dim = dim;
  v->dr = dr[id];
  v->pass = n_adjust;
  for (int d = 0; d < 3; ++d) {
    v->ix[d] = d < dim ? ix[(size_t)id * dim + d] : 0;
    v->r_min[d] = d < dim ? r_min[(size_t)id * dim + d] : 0.0;
  }
}

// consistent_ref_flags, core:628-725
int HostTree::consistent_flags(std::vector<int>& flags, afv_ref_fn fn, void* user,
                               std::string& err) {
  std::fill(flags.begin(), flags.end(), (int)kKeepRef);
  afv_box_view v;
  for (int l = 1; l <= highest_lvl; ++l) {
    for (int id : L(l).leaves) {
      make_view(id, &v);
      fn(&v, &flags[id], user);
      int p = parent[id];
      if (p > kNoBox && ichild_of(id) == 1) {
        make_view(p, &v);
        fn(&v, &flags[p], user);
      }
    }
  }
  for (size_t i = 1; i < flags.size(); ++i)
    if (flags[i] > kDoRef || flags[i] < kRmRef) return err = "invalid refinement flag given", AFV_ERR_INVALID;

  for (int id : L(lvl_limit).ids)  // no refinement beyond lvl_limit
    if (flags[id] == kDoRef) flags[id] = kKeepRef;

  // 2:1 balance, finest level first.
  for (int l = highest_lvl; l >= 1; --l) {
    for (int id : L(l).leaves) {
      if (flags[id] > kKeepRef) {
        flags[id] = kRefine;
        for (int nb = 0; nb < nnb; ++nb)
          if (neighbors[(size_t)id * nnb + nb] == kNoBox) {
            int p_nb = neighbors[(size_t)parent[id] * nnb + nb];
            flags[p_nb] = kRefine;
          }
      } else if (flags[id] == kRmRef) {
        for (int nb = 0; nb < nnb; ++nb) {
          int n_id = neighbors[(size_t)id * nnb + nb];
          if (n_id > kNoBox && (has_children(n_id) || flags[n_id] > kKeepRef)) {
            flags[id] = kKeepRef;
            break;
          }
        }
      }
    }
  }
  // A parent is derefined only if all its children ask for it and it does
  // not itself ask for refinement; at most one level goes per call.
  for (int l = highest_lvl - 1; l >= 1; --l) {
    for (int id : L(l).parents) {
      bool all_rm = true;
      for (int c = 0; c < nch; ++c)
        if (flags[children[(size_t)id * nch + c]] != kRmRef) all_rm = false;
      flags[id] = (all_rm && flags[id] <= kKeepRef) ? kDerefine : kKeepRef;
    }
  }
  return AFV_OK;
}

void HostTree::add_children(int id, const int* c_ids) {  // core:752-787
  for (int c = 0; c < nch; ++c) children[(size_t)id * nch + c] = c_ids[c];
  for (int c = 0; c < nch; ++c) {
    int k = c_ids[c];
    for (int d = 0; d < dim; ++d) {
      int bit = child_bit(c, d);
      ix[(size_t)k * dim + d] = 2 * ix[(size_t)id * dim + d] - 1 + bit;
      r_min[(size_t)k * dim + d] = r_min[(size_t)id * dim + d] + 0.5 * dr[id] * bit * ncell[id];
    }
    lvl[k] = lvl[id] + 1;
    parent[k] = id;
    std::fill_n(&children[(size_t)k * nch], nch, kNoBox);
    std::fill_n(&neighbors[(size_t)k * nnb], nnb, kNoBox);
    ncell[k] = ncell[id];
    dr[k] = 0.5 * dr[id];
    in_use[k] = 1;
  }
  // Physical boundaries are inherited by the children on that side.
  for (int nb = 0; nb < nnb; ++nb) {
    int v = neighbors[(size_t)id * nnb + nb];
    if (v < kNoBox) {
      int d = nb >> 1, h = nb & 1;
      for (int c = 0; c < nch; ++c)
        if (child_bit(c, d) == h) neighbors[(size_t)c_ids[c] * nnb + nb] = v;
    }
  }
}

void HostTree::remove_children(int id) {  // core:728-749
  for (int c = 0; c < nch; ++c) {
    int k = children[(size_t)id * nch + c];
    for (int nb = 1; nb <= nnb; ++nb) {
      int v = neighbors[(size_t)k * nnb + nb - 1];
      if (v > kNoBox) neighbors[(size_t)v * nnb + nb_rev(nb) - 1] = kNoBox;
    }
    in_use[k] = 0;
  }
  std::fill_n(&children[(size_t)id * nch], nch, kNoBox);
}

// find_neighb_$Dd, core:404-422: through the parent, or the parent's neighbour
// when the box sits on the same side as the requested neighbour.
int HostTree::find_neighb(int id, int nb1) const {
  int p = parent[id];
  int c0 = ichild_of(id) - 1;
  int d = nb_dim(nb1);
  bool low_child = child_bit(c0, d) == 0;
  bool low_nb = nb_high(nb1) == 0;
  if (low_child == low_nb) p = neighbors[(size_t)p * nnb + nb1 - 1];
  return children[(size_t)p * nch + (c0 ^ (1 << d))];
}

void HostTree::set_neighbs(int id) {  // core:387-401
  for (int nb1 = 1; nb1 <= nnb; ++nb1) {
    if (neighbors[(size_t)id * nnb + nb1 - 1] != kNoBox) continue;
    int v = find_neighb(id, nb1);
    if (v > kNoBox) {
      neighbors[(size_t)id * nnb + nb1 - 1] = v;
      neighbors[(size_t)v * nnb + nb_rev(nb1) - 1] = id;
    }
  }
}

// a$D_adjust_refinement, core:452-541
int HostTree::adjust(afv_ref_fn fn, void* user, int* n_add, int* n_rm, std::string& err) {
  if (!ready) return err = "tree not ready (call set_base first)", AFV_ERR_STATE;
  if (!fn) return err = "no refinement function", AFV_ERR_INVALID;
  tidy_up(0.5, 1000);
  int prev = highest_id;
  std::vector<int> flags((size_t)prev + 1, kKeepRef);
  int rc = consistent_flags(flags, fn, user, err);
  if (rc) return rc;
  n_adjust++;
  int n_ref = 0, n_drf = 0;
  for (int id = 1; id <= prev; ++id) {
    n_ref += flags[id] == kRefine;
    n_drf += flags[id] == kDerefine;
  }
  int n_new = nch * n_ref;
  if ((long long)n_used() + n_new > box_limit) {
    err = "exceeding memory limit (box_limit " + std::to_string(box_limit) + ")";
    return AFV_ERR_BUDGET;
  }
  if (prev + n_new > capacity()) resize(2 * (prev + n_new));

  int l = 1;
  for (; l <= lvl_limit - 1; ++l) {
    LevelLists& lv = L(l);
    for (size_t i = 0; i < lv.ids.size(); ++i) {
      int id = lv.ids[i];
      if (id > prev) continue;
      if (flags[id] == kRefine) {
        int c_ids[8];
        get_free_ids(nch, c_ids);
        add_children(id, c_ids);
      } else if (flags[id] == kDerefine) {
        remove_children(id);
      }
    }
    lists_of(lv);
    LevelLists& up = L(l + 1);
    up.ids.clear();
    for (int p : lv.parents)
      for (int c = 0; c < nch; ++c) up.ids.push_back(children[(size_t)p * nch + c]);
    for (int id : up.ids)
      if (id > prev) set_neighbs(id);
    if (up.ids.empty()) break;
  }
  if (l > lvl_limit - 1) l = lvl_limit;
  highest_lvl = l;
  lists_of(L(highest_lvl + 1));
  if (n_add) *n_add = nch * n_ref;
  if (n_rm) *n_rm = nch * n_drf;
  return AFV_OK;
}

// ---------------------------------------------------------------------------
// Built-in criteria and sources
// ---------------------------------------------------------------------------

double source_eval(int dim, int lpl, const double* g, int n_gauss, const double* r) {
  double s = 0;
  for (int k = 0; k < n_gauss; ++k) {
    const double* p = g + (size_t)k * (2 + dim);
    double xr2 = 0;
    for (int d = 0; d < dim; ++d) {
      double x = (r[d] - p[2 + d]) / p[1];
      xr2 = xr2 + x * x;
    }
    if (lpl)
      s = s + p[0] * (4 / (p[1] * p[1]) * (xr2 - 0.5 * dim) * std::exp(-xr2));
    else
      s = s + p[0] * std::exp(-xr2);
  }
  return s;
}

void builtin_ref_fn(const afv_box_view* b, int* flag, void* user) {
  const BuiltinCrit* bc = static_cast<const BuiltinCrit*>(user);
  const afv_ref_crit& c = bc->c;
  int dim = b->dim;
  switch (c.kind) {
    case AFV_REF_UNIFORM:
      if (b->lvl < c.lvl_max) *flag = AFV_DO_REF;
      return;
    case AFV_REF_SOURCE: {
      if (b->lvl >= c.lvl_max) return;
      int nc = b->n_cell;
      double dr2 = b->dr * b->dr;
      int kmax = dim == 3 ? nc : 1;
      for (int k = 1; k <= kmax; ++k)
        for (int j = 1; j <= nc; ++j)
          for (int i = 1; i <= nc; ++i) {
            int cix[3] = {i, j, k};
            double r[3];
            for (int d = 0; d < dim; ++d) r[d] = b->r_min[d] + (cix[d] - 0.5) * b->dr;
            double f = source_eval(dim, c.src_lpl, bc->gauss.data(), c.n_gauss, r);
            if (std::fabs(f) * dr2 > c.thr) {
              *flag = AFV_DO_REF;
              return;
            }
          }
      return;
    }
    case AFV_REF_RANDOM:
    case AFV_REF_RANDOM_RM: {
      // Uniform [0,1) keyed by (seed, pass, lvl, ix): independent of the order
      // in which boxes are visited.
      uint64_t h = mix(c.seed ^ 0xA5A5A5A5ull);
      h = mix(h ^ (uint64_t)(uint32_t)b->pass);
      h = mix(h ^ (uint64_t)(uint32_t)b->lvl);
      for (int d = 0; d < dim; ++d) h = mix(h ^ (uint64_t)(uint32_t)b->ix[d]);
      double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
      if (u < c.prob && b->lvl < c.lvl_max)
        *flag = AFV_DO_REF;
      else if (c.kind == AFV_REF_RANDOM_RM)
        *flag = AFV_RM_REF;
      return;
    }
  }
}

}  // namespace afv
