#include "plan.hpp"

#include <algorithm>
#include <cstring>
#include <numeric>

namespace afv {

namespace {
long long ipow(int b, int e) {
  long long r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}
}  // namespace

int build_plan(const std::vector<const HostTree*>& trees, Plan& p, std::string& err) {
  if (trees.empty()) return err = "no trees", AFV_ERR_INVALID;
  const HostTree& t0 = *trees[0];
  p = Plan();
  p.dim = t0.dim;
  p.nc = t0.n_cell;
  p.min_lvl = t0.min_lvl;
  p.cyl = t0.coord == 1;
  p.n_trees = (int)trees.size();
  const int D = p.dim, NCH = 1 << D, NNB = 2 * D;
  int max_lvl = 1;
  for (const HostTree* t : trees) {
    if (!t->ready) return err = "tree without base (set_base not called)", AFV_ERR_STATE;
    if (t->dim != D || t->n_cell != p.nc || t->min_lvl != p.min_lvl || t->coord != t0.coord)
      return err = "trees of one forest need the same dim, n_cell, coarsen_to and coordinates", AFV_ERR_INVALID;
    max_lvl = std::max(max_lvl, t->highest_lvl);
  }
  p.max_lvl = max_lvl;
  if (D == 2 && !(p.nc == 4 || p.nc == 8 || p.nc == 16))
    return err = "2-D boxes of 4, 8 or 16 cells per direction are supported", AFV_ERR_UNSUPPORTED;
  if (D == 3 && !(p.nc == 4 || p.nc == 8))
    return err = "3-D boxes of 4 or 8 cells per direction are supported", AFV_ERR_UNSUPPORTED;
  if (p.nc_at(p.min_lvl) < 2) return err = "coarsest boxes need >= 2 cells", AFV_ERR_UNSUPPORTED;

  const int nlev = max_lvl - p.min_lvl + 1;
  p.lvl_lo.assign(nlev, 0);
  p.lvl_n.assign(nlev, 0);
  p.leaves.assign(nlev, {});
  p.parents.assign(nlev, {});
  p.host_order.assign(p.n_trees, {});
  p.tree_highest.assign(p.n_trees, 0);
  p.tree_leaf_cells.assign(p.n_trees, 0);
  p.bc.assign(p.n_trees, BcSpec());

  // slot_of[t][id]
  std::vector<std::vector<int>> slot_of(p.n_trees);
  for (int t = 0; t < p.n_trees; ++t) slot_of[t].assign((size_t)trees[t]->highest_id + 1, -1);

  int s = 0;
  for (int l = p.min_lvl; l <= max_lvl; ++l) {
    p.lvl_lo[p.L(l)] = s;
    for (int t = 0; t < p.n_trees; ++t) {
      const HostTree& T = *trees[t];
      if (l > T.highest_lvl) continue;
      std::vector<int> ids = T.L(l).ids;
      std::vector<uint64_t> key(ids.size());
      for (size_t n = 0; n < ids.size(); ++n) {
        int ix0[3] = {0, 0, 0};
        for (int d = 0; d < D; ++d) ix0[d] = T.ix[(size_t)ids[n] * D + d] - 1;
        key[n] = morton_key(D, ix0);
      }
      std::vector<int> perm(ids.size());
      std::iota(perm.begin(), perm.end(), 0);
      std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
      for (int k : perm) {
        int id = ids[k];
        if (id < 1 || id > T.highest_id || !T.in_use[id] || T.lvl[id] != l)
          return err = "level list holds an invalid box id", AFV_ERR_INVALID;
        if (slot_of[t][id] >= 0) return err = "box listed twice", AFV_ERR_INVALID;
        slot_of[t][id] = s++;
      }
    }
    p.lvl_n[p.L(l)] = s - p.lvl_lo[p.L(l)];
  }
  p.n_slots = s;
  const int N = s;
  p.nb.assign((size_t)N * NNB, 0);
  p.parent.assign(N, -1);
  p.first_child.assign(N, -1);
  p.tree.assign(N, 0);
  p.lvl.assign(N, 0);
  p.qd.assign(N, -1);
  p.host_id.assign(N, 0);
  p.ix.assign((size_t)N * D, 0);
  p.dr.assign(N, 0);
  p.r_min.assign((size_t)N * D, 0);
  p.offg.assign(N, 0);
  p.offi.assign(N, 0);
  p.bctype.assign((size_t)N * NNB, 0);
  p.bcoff.assign((size_t)N * NNB, -1);

  long long og = 0, oi = 0;
  for (int t = 0; t < p.n_trees; ++t) p.tree_highest[t] = trees[t]->highest_lvl;
  for (int t = 0; t < p.n_trees; ++t) {
    const HostTree& T = *trees[t];
    for (int l = T.min_lvl; l <= T.highest_lvl; ++l)
      for (int id : T.L(l).ids) p.host_order[t].push_back(slot_of[t][id]);
  }
  for (int l = p.min_lvl; l <= max_lvl; ++l) {
    const int nc_l = p.nc_at(l);
    const long long sg = ipow(nc_l + 2, D), si = ipow(nc_l, D);
    for (int k = 0; k < p.lvl_n[p.L(l)]; ++k) {
      int sl = p.lvl_lo[p.L(l)] + k;
      p.offg[sl] = og;
      p.offi[sl] = oi;
      og += sg;
      oi += si;
    }
  }
  p.n_elem_g = og;
  p.n_elem_i = oi;

  for (int t = 0; t < p.n_trees; ++t) {
    const HostTree& T = *trees[t];
    for (int id = 1; id <= T.highest_id; ++id) {
      int sl = slot_of[t][id];
      if (sl < 0) continue;
      int l = T.lvl[id];
      p.tree[sl] = t;
      p.lvl[sl] = l;
      p.host_id[sl] = id;
      p.dr[sl] = T.dr[id];
      if (T.ncell[id] != p.nc_at(l)) return err = "box n_cell does not match its level", AFV_ERR_INVALID;
      for (int d = 0; d < D; ++d) {
        p.ix[(size_t)sl * D + d] = T.ix[(size_t)id * D + d];
        p.r_min[(size_t)sl * D + d] = T.r_min[(size_t)id * D + d];
      }
      int par = T.parent[id];
      if (l > p.min_lvl) {
        if (par < 1 || par > T.highest_id || slot_of[t][par] < 0 || T.lvl[par] != l - 1)
          return err = "box without a valid parent", AFV_ERR_INVALID;
        p.parent[sl] = slot_of[t][par];
      } else if (par != 0) {
        return err = "coarsest box with a parent", AFV_ERR_INVALID;
      }
      if (l >= 2) {
        int q = 0;
        for (int d = 0; d < D; ++d) q |= ((T.ix[(size_t)id * D + d] - 1) & 1) << d;
        p.qd[sl] = q;
      }
      // children: all 2^D for levels >= 1, only the first one below
      const int* ch = &T.children[(size_t)id * NCH];
      if (ch[0] != kNoBox) {
        int c0 = (ch[0] >= 1 && ch[0] <= T.highest_id) ? slot_of[t][ch[0]] : -1;
        if (c0 < 0) return err = "child box not in the level lists", AFV_ERR_INVALID;
        p.first_child[sl] = c0;
        int nchild = l >= 1 ? NCH : 1;
        for (int c = 0; c < nchild; ++c) {
          int cs = (ch[c] >= 1 && ch[c] <= T.highest_id) ? slot_of[t][ch[c]] : -1;
          if (cs != c0 + c) return err = "children are not a complete Morton family", AFV_ERR_INVALID;
          if (T.parent[ch[c]] != id) return err = "child/parent links disagree", AFV_ERR_INVALID;
        }
        for (int c = nchild; c < NCH; ++c)
          if (ch[c] != kNoBox) return err = "sub-level box with more than one child", AFV_ERR_INVALID;
      }
      for (int f = 0; f < NNB; ++f) {
        int v = T.neighbors[(size_t)id * NNB + f];
        int code;
        if (v > 0) {
          if (v > T.highest_id || slot_of[t][v] < 0 || T.lvl[v] != l)
            return err = "neighbour box not on the same level", AFV_ERR_INVALID;
          code = slot_of[t][v];
        } else if (v == 0) {
          // Refinement boundary: needs a parent whose neighbour in this
          // direction exists (2:1 balance), see mg$D_sides_rb.
          if (l < 2) return err = "refinement boundary below level 2", AFV_ERR_INVALID;
          int pnb = T.neighbors[(size_t)par * NNB + f];
          if (pnb <= 0) return err = "refinement boundary without a coarse neighbour", AFV_ERR_INVALID;
          if (T.children[(size_t)id * NCH] != kNoBox)
            return err = "refined box at a refinement boundary (tree not 2:1 balanced)", AFV_ERR_INVALID;
          code = -1;
        } else {
          code = -2;
        }
        p.nb[(size_t)sl * NNB + f] = code;
      }
    }
  }
  // Offsets of the box each ghost face reads from.
  p.nbo.assign((size_t)N * NNB, -1);
  for (int sl = 0; sl < N; ++sl)
    for (int f = 0; f < NNB; ++f) {
      int code = p.nb[(size_t)sl * NNB + f];
      if (code >= 0)
        p.nbo[(size_t)sl * NNB + f] = p.offg[code];
      else if (code == -1)
        p.nbo[(size_t)sl * NNB + f] = p.offg[p.parent[sl]];
    }
  // per-level leaf / parent lists in slot order
  for (int l = p.min_lvl; l <= max_lvl; ++l) {
    for (int k = 0; k < p.lvl_n[p.L(l)]; ++k) {
      int sl = p.lvl_lo[p.L(l)] + k;
      if (p.first_child[sl] >= 0)
        p.parents[p.L(l)].push_back(sl);
      else {
        p.leaves[p.L(l)].push_back(sl);
        if (l < 1) return err = "leaf below level 1", AFV_ERR_UNSUPPORTED;
        p.all_leaves.push_back(sl);
        p.tree_leaf_cells[p.tree[sl]] += ipow(p.nc, D);
      }
    }
  }
  // all leaves tree by tree (levels, then slots, within a tree), and the
  // counts over leading trees
  std::stable_sort(p.all_leaves.begin(), p.all_leaves.end(),
                   [&](int a, int b) { return p.tree[a] < p.tree[b]; });
  const int T1 = p.n_trees + 1;
  p.lvl_tprefix.assign((size_t)nlev * T1, 0);
  p.leaves_tprefix.assign((size_t)nlev * T1, 0);
  p.parents_tprefix.assign((size_t)nlev * T1, 0);
  p.all_leaves_tprefix.assign(T1, 0);
  for (int L = 0; L < nlev; ++L) {
    int* lv = &p.lvl_tprefix[(size_t)L * T1];
    for (int k = 0; k < p.lvl_n[L]; ++k) ++lv[p.tree[p.lvl_lo[L] + k] + 1];
    int* le = &p.leaves_tprefix[(size_t)L * T1];
    for (int sl : p.leaves[L]) ++le[p.tree[sl] + 1];
    int* pa = &p.parents_tprefix[(size_t)L * T1];
    for (int sl : p.parents[L]) ++pa[p.tree[sl] + 1];
    for (int t = 0; t < p.n_trees; ++t) {
      lv[t + 1] += lv[t];
      le[t + 1] += le[t];
      pa[t + 1] += pa[t];
    }
  }
  for (int sl : p.all_leaves) ++p.all_leaves_tprefix[p.tree[sl] + 1];
  for (int t = 0; t < p.n_trees; ++t) p.all_leaves_tprefix[t + 1] += p.all_leaves_tprefix[t];
  for (int t = 0; t < p.n_trees; ++t) plan_fill_bc(p, t);
  plan_build_desc(p);
  return AFV_OK;
}

void plan_count_bc_faces(const Plan& p, int t, long long& n_faces, long long& n_values) {
  const int D = p.dim, NNB = 2 * D;
  n_faces = n_values = 0;
  for (int s : p.host_order[t])
    for (int f = 0; f < NNB; ++f)
      if (p.nb[(size_t)s * NNB + f] == -2) {
        int ncl = p.nc_at(p.lvl[s]);
        ++n_faces;
        n_values += D == 2 ? ncl : (long long)ncl * ncl;
      }
}

void plan_fill_bc(Plan& p, int t) {
  const int D = p.dim, NNB = 2 * D;
  const BcSpec& bc = p.bc[t];
  // Caller-given records: position of each face in the caller's lists.
  std::vector<long long> face_pos, val_pos;
  if (bc.per_face) {
    face_pos.assign(p.nb.size(), -1);
    val_pos.assign(p.nb.size(), -1);
    long long nf = 0, nv = 0;
    for (int s : p.host_order[t])
      for (int f = 0; f < NNB; ++f) {
        size_t k = (size_t)s * NNB + f;
        if (p.nb[k] != -2) continue;
        int ncl = p.nc_at(p.lvl[s]);
        face_pos[k] = nf++;
        val_pos[k] = nv;
        nv += D == 2 ? ncl : (long long)ncl * ncl;
      }
  }
  // Rebuild the value table: other trees' records are kept, this tree's
  // records are recomputed from its BcSpec.
  std::vector<double> vals;
  std::vector<long long> newoff(p.bcoff.size(), -1);
  for (int s = 0; s < p.n_slots; ++s)
    for (int f = 0; f < NNB; ++f) {
      size_t k = (size_t)s * NNB + f;
      if (p.nb[k] != -2) continue;
      if (p.tree[s] != t) {
        if (p.bcoff[k] >= 0) {
          int ncl = p.nc_at(p.lvl[s]);
          long long nfc = D == 2 ? ncl : (long long)ncl * ncl;
          newoff[k] = (long long)vals.size();
          vals.insert(vals.end(), p.bcval.begin() + p.bcoff[k], p.bcval.begin() + p.bcoff[k] + nfc);
        }
        continue;
      }
      if (bc.per_face) {
        int ncl = p.nc_at(p.lvl[s]);
        long long nfc = D == 2 ? ncl : (long long)ncl * ncl;
        p.bctype[k] = bc.face_type[face_pos[k]] == AFV_BC_NEUMANN ? 1 : 0;
        newoff[k] = (long long)vals.size();
        vals.insert(vals.end(), bc.face_vals.begin() + val_pos[k],
                    bc.face_vals.begin() + val_pos[k] + nfc);
        continue;
      }
      p.bctype[k] = bc.type == AFV_BC_NEUMANN ? 1 : 0;
      if (bc.gauss.empty()) continue;
      int ncl = p.nc_at(p.lvl[s]);
      int dim = f >> 1;
      bool low = (f & 1) == 0;
      newoff[k] = (long long)vals.size();
      int cmax = D == 3 ? ncl : 1;
      for (int c = 1; c <= cmax; ++c)
        for (int a = 1; a <= ncl; ++a) {
          // face centre: a$D_rr_cc(box, [0.5 or nc+0.5, tangential indices])
          int tang[2] = {a, c};
          int k2 = 0;
          double r[3];
          for (int e = 0; e < D; ++e) {
            double cix = (e == dim) ? (low ? 0.5 : ncl + 0.5) : (double)tang[k2++];
            r[e] = p.r_min[(size_t)s * D + e] + (cix - 0.5) * p.dr[s];
          }
          vals.push_back(source_eval(D, bc.src_lpl, bc.gauss.data(),
                                     (int)bc.gauss.size() / (2 + D), r));
        }
    }
  p.bcval.swap(vals);
  p.bcoff.swap(newoff);
}

void plan_build_desc(Plan& p) {
  const int NNB = 2 * p.dim;
  p.desc.assign(p.n_slots, SlotDesc());
  for (int s = 0; s < p.n_slots; ++s) {
    SlotDesc& d = p.desc[s];
    std::memset(&d, 0, sizeof(d));
    for (int f = 0; f < 6; ++f) {
      d.code[f] = kFaceDirichlet;
      d.nbo[f] = -1;
    }
    for (int f = 0; f < NNB; ++f) {
      size_t k = (size_t)s * NNB + f;
      int code = p.nb[k];
      if (code >= 0) {
        d.code[f] = 0;
        d.nbo[f] = p.nbo[k];
      } else if (code == -1) {
        d.code[f] = kFaceRefinement;
        d.nbo[f] = p.nbo[k];
      } else {
        d.code[f] = p.bctype[k] ? kFaceNeumann : kFaceDirichlet;
        d.nbo[f] = p.bcoff[k];
      }
    }
    d.qd = p.qd[s];
    d.tree = p.tree[s];
    d.dr = p.dr[s];
    d.dx2 = p.dr[s] * p.dr[s];
    d.inv_dx2 = 1 / (p.dr[s] * p.dr[s]);
    d.offg = p.offg[s];
    d.offi = p.offi[s];
    d.drf = (float)p.dr[s];
    d.dx2f = (float)(p.dr[s] * p.dr[s]);
    d.inv_dx2f = 1.0f / (float)(p.dr[s] * p.dr[s]);
    d.first_child = p.first_child[s];
    d.parent = p.parent[s];
  }
  // Two-hop sources for refinement boundaries: the parent's neighbour in the
  // face direction, whose boundary cells the parent's ghost cells copy.
  p.nbo2.assign((size_t)p.n_slots * NNB, -1);
  for (int s = 0; s < p.n_slots; ++s)
    for (int f = 0; f < NNB; ++f)
      if (p.nb[(size_t)s * NNB + f] == -1) {
        int par = p.parent[s];
        int q = p.nb[(size_t)par * NNB + f];
        if (q >= 0) p.nbo2[(size_t)s * NNB + f] = p.offg[q];
      }
}

}  // namespace afv
