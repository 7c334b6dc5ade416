// extern "C" boundary of the library (declared in include/afivo_gb300.h).
// Every entry point validates its arguments, never aborts, and reports
// failures through a status code and afv_last_error().
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "afivo_gb300.h"
#include "forest.hpp"
#include "host_tree.hpp"

struct afv_tree {
  afv::HostTree t;
};
struct afv_forest {
  afv::Forest f;
};

namespace afv {
class DevTree;
int dtree_create(const HostTree& h, int device, DevTree** out, std::string& err);
void dtree_destroy(DevTree* t);
int dtree_adjust(DevTree* t, const afv_ref_crit* c, int* n_add, int* n_rm, std::string& err);
int dtree_download(const DevTree* t, HostTree& h, std::string& err);
int dtree_info(const DevTree* t, int* out5);
}  // namespace afv

struct afv_dtree {
  afv::DevTree* t = nullptr;
  ~afv_dtree() {
    if (t) afv::dtree_destroy(t);
  }
};

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    std::string err;
    int rc = f(err);
    if (rc != AFV_OK) g_err = err.empty() ? "error" : err;
    return rc;
  } catch (const std::bad_alloc&) {
    return fail(AFV_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(AFV_ERR_INVALID, e.what());
  }
}

afv::MgOpts mg_of(const afv_mg_opts* o) {
  afv::MgOpts m;
  if (o) {
    m.n_down = o->n_cycle_down < 0 ? 2 : o->n_cycle_down;
    m.n_up = o->n_cycle_up < 0 ? 2 : o->n_cycle_up;
    m.n_base = o->n_cycle_base < 0 ? 2 : o->n_cycle_base;
  }
  return m;
}
}  // namespace

namespace afv {
int forest_add_vars(Forest& F, int n_cc, int n_fc, std::string& err);
int forest_fc_exchange(Forest& F, int t, int ifc, double* host, bool to_dev, std::string& err);
long long forest_fc_count(const Forest& F, int t);
int forest_prolong(Forest& F, int lp, int iv, int iv_to, int order, int add, std::string& err);
int forest_restrict_tree(Forest& F, int iv, int iv_to, std::string& err);
int forest_gc_tree_var(Forest& F, int iv, int rb, int bc, std::string& err);
int forest_gc2_level(Forest& F, int tree, int lvl, int iv, double* host_out, long long n_out, std::string& err);
int forest_consistent_fluxes(Forest& F, int n, const int* f_ixs, std::string& err);
int forest_write_vtk(Forest& F, int tree, const char* filename, int n_cycle, double time, int n_cc, const int* ixs_cc,
                     const char* const* cc_names, int n_fcv, const int* ixs_fc, const char* const* fc_names,
                     const char* dir, std::string& err);
}  // namespace afv

extern "C" {

const char* afv_last_error(void) { return g_err.c_str(); }
int afv_version(void) { return 1; }

int afv_tree_create(int dim, int n_cell, double dr, const double* r_min, int lvl_limit,
                    int coarsen_to, double mem_limit_gb, afv_tree** out) {
  if (!out) return fail(AFV_ERR_INVALID, "out is NULL");
  *out = nullptr;
  return guarded([&](std::string& err) -> int {
    std::unique_ptr<afv_tree> t(new afv_tree());
    int rc = t->t.init(dim, n_cell, dr, r_min, lvl_limit, coarsen_to, mem_limit_gb, err);
    if (rc) return rc;
    *out = t.release();
    return AFV_OK;
  });
}

int afv_tree_set_coord(afv_tree* t, int coord) {
  if (!t) return fail(AFV_ERR_INVALID, "tree is NULL");
  if (coord != AFV_COORD_XYZ && coord != AFV_COORD_CYL) return fail(AFV_ERR_INVALID, "unknown coordinate system");
  if (coord == AFV_COORD_CYL && t->t.dim != 2) return fail(AFV_ERR_INVALID, "cylindrical coordinates need a 2-D tree");
  t->t.coord = coord;
  return AFV_OK;
}

int afv_tree_set_base(afv_tree* t, int n_boxes, const int* ix_list, const int* nb_list) {
  if (!t || !ix_list || !nb_list) return fail(AFV_ERR_INVALID, "NULL argument");
  return guarded([&](std::string& err) -> int {
    std::vector<int> nb(nb_list, nb_list + (size_t)n_boxes * t->t.nnb);
    return t->t.set_base(n_boxes, ix_list, nb.data(), err);
  });
}

int afv_tree_adjust_refinement(afv_tree* t, afv_ref_fn fn, void* user, int* n_add, int* n_rm) {
  if (!t) return fail(AFV_ERR_INVALID, "tree is NULL");
  return guarded([&](std::string& err) -> int { return t->t.adjust(fn, user, n_add, n_rm, err); });
}

int afv_tree_adjust_builtin(afv_tree* t, const afv_ref_crit* crit, int* n_add, int* n_rm) {
  if (!t || !crit) return fail(AFV_ERR_INVALID, "NULL argument");
  if (crit->kind < AFV_REF_UNIFORM || crit->kind > AFV_REF_RANDOM_RM)
    return fail(AFV_ERR_INVALID, "unknown refinement criterion");
  if (crit->kind == AFV_REF_SOURCE && (crit->n_gauss <= 0 || !crit->gauss))
    return fail(AFV_ERR_INVALID, "source criterion needs Gaussians");
  return guarded([&](std::string& err) -> int {
    afv::BuiltinCrit bc;
    bc.c = *crit;
    bc.dim = t->t.dim;
    bc.tree = &t->t;
    if (crit->n_gauss > 0 && crit->gauss)
      bc.gauss.assign(crit->gauss, crit->gauss + (size_t)crit->n_gauss * (2 + t->t.dim));
    return t->t.adjust(afv::builtin_ref_fn, &bc, n_add, n_rm, err);
  });
}

int afv_tree_refine_builtin(afv_tree* t, const afv_ref_crit* crit, int max_passes, int* n_passes) {
  int passes = 0;
  for (; passes < max_passes; ++passes) {
    int na = 0, nr = 0;
    int rc = afv_tree_adjust_builtin(t, crit, &na, &nr);
    if (rc) return rc;
    if (na == 0) {
      ++passes;
      break;
    }
  }
  if (n_passes) *n_passes = passes;
  return AFV_OK;
}

void afv_tree_destroy(afv_tree* t) { delete t; }

int afv_dtree_create(const afv_tree* t, int device, afv_dtree** out) {
  if (!t || !out) return fail(AFV_ERR_INVALID, "NULL argument");
  *out = nullptr;
  return guarded([&](std::string& err) -> int {
    std::unique_ptr<afv_dtree> d(new afv_dtree());
    if (int rc = afv::dtree_create(t->t, device, &d->t, err)) return rc;
    *out = d.release();
    return AFV_OK;
  });
}

void afv_dtree_destroy(afv_dtree* t) { delete t; }

int afv_dtree_adjust_builtin(afv_dtree* t, const afv_ref_crit* crit, int* n_add, int* n_rm) {
  if (!t || !crit) return fail(AFV_ERR_INVALID, "NULL argument");
  if (crit->kind == AFV_REF_SOURCE && (crit->n_gauss <= 0 || !crit->gauss))
    return fail(AFV_ERR_INVALID, "source criterion needs Gaussians");
  return guarded([&](std::string& err) -> int { return afv::dtree_adjust(t->t, crit, n_add, n_rm, err); });
}

int afv_dtree_refine_builtin(afv_dtree* t, const afv_ref_crit* crit, int max_passes, int* n_passes) {
  int passes = 0;
  for (; passes < max_passes; ++passes) {
    int na = 0, nr = 0;
    int rc = afv_dtree_adjust_builtin(t, crit, &na, &nr);
    if (rc) return rc;
    if (na == 0) {
      ++passes;
      break;
    }
  }
  if (n_passes) *n_passes = passes;
  return AFV_OK;
}

int afv_dtree_download(const afv_dtree* t, afv_tree* host) {
  if (!t || !host) return fail(AFV_ERR_INVALID, "NULL argument");
  return guarded([&](std::string& err) -> int { return afv::dtree_download(t->t, host->t, err); });
}

int afv_dtree_get_info(const afv_dtree* t, int* out5) {
  if (!t || !out5) return fail(AFV_ERR_INVALID, "NULL argument");
  return afv::dtree_info(t->t, out5);
}

int afv_tree_get_info(const afv_tree* t, int* out8) {
  if (!t || !out8) return fail(AFV_ERR_INVALID, "NULL argument");
  const afv::HostTree& h = t->t;
  int leaves = 0;
  if (h.ready)
    for (int l = h.min_lvl; l <= h.highest_lvl; ++l) leaves += (int)h.L(l).leaves.size();
  out8[0] = h.dim;
  out8[1] = h.n_cell;
  out8[2] = h.min_lvl;
  out8[3] = h.highest_lvl;
  out8[4] = h.highest_id;
  out8[5] = h.ready ? h.n_used() : 0;
  out8[6] = leaves;
  out8[7] = h.lvl_limit;
  return AFV_OK;
}

int afv_tree_export(const afv_tree* t, int* lvl, int* ix, int* parent, int* children,
                    int* neighbors, int* n_cell, double* dr, double* r_min, int* in_use) {
  if (!t) return fail(AFV_ERR_INVALID, "tree is NULL");
  const afv::HostTree& h = t->t;
  for (int id = 1; id <= h.highest_id; ++id) {
    int k = id - 1;
    if (lvl) lvl[k] = h.lvl[id];
    if (parent) parent[k] = h.parent[id];
    if (n_cell) n_cell[k] = h.ncell[id];
    if (dr) dr[k] = h.dr[id];
    if (in_use) in_use[k] = h.in_use[id];
    for (int d = 0; d < h.dim; ++d) {
      if (ix) ix[k * h.dim + d] = h.ix[(size_t)id * h.dim + d];
      if (r_min) r_min[k * h.dim + d] = h.r_min[(size_t)id * h.dim + d];
    }
    for (int c = 0; c < h.nch; ++c)
      if (children) children[k * h.nch + c] = h.children[(size_t)id * h.nch + c];
    for (int nb = 0; nb < h.nnb; ++nb)
      if (neighbors) neighbors[k * h.nnb + nb] = h.neighbors[(size_t)id * h.nnb + nb];
  }
  return AFV_OK;
}

int afv_tree_level(const afv_tree* t, int lvl, int* sizes3, int* ids, int* leaves, int* parents) {
  if (!t || !sizes3) return fail(AFV_ERR_INVALID, "NULL argument");
  const afv::HostTree& h = t->t;
  if (lvl < h.min_lvl || lvl > h.lvl_limit + 1) return fail(AFV_ERR_INVALID, "level out of range");
  const afv::LevelLists& L = h.L(lvl);
  sizes3[0] = (int)L.ids.size();
  sizes3[1] = (int)L.leaves.size();
  sizes3[2] = (int)L.parents.size();
  if (ids) std::memcpy(ids, L.ids.data(), L.ids.size() * sizeof(int));
  if (leaves) std::memcpy(leaves, L.leaves.data(), L.leaves.size() * sizeof(int));
  if (parents) std::memcpy(parents, L.parents.data(), L.parents.size() * sizeof(int));
  return AFV_OK;
}

int afv_forest_create(int n_trees, afv_tree* const* trees, const afv_forest_opts* opts,
                      afv_forest** out) {
  if (!out || !trees || n_trees <= 0) return fail(AFV_ERR_INVALID, "bad arguments");
  *out = nullptr;
  return guarded([&](std::string& err) -> int {
    std::vector<const afv::HostTree*> v;
    for (int i = 0; i < n_trees; ++i) {
      if (!trees[i]) return err = "NULL tree", AFV_ERR_INVALID;
      v.push_back(&trees[i]->t);
    }
    std::unique_ptr<afv_forest> f(new afv_forest());
    int rc = f->f.create(v, opts, err);
    if (rc) return rc;
    *out = f.release();
    return AFV_OK;
  });
}

void afv_forest_destroy(afv_forest* f) { delete f; }

int afv_forest_get_info(const afv_forest* f, long long* out8) {
  if (!f || !out8) return fail(AFV_ERR_INVALID, "NULL argument");
  const afv::Plan& p = f->f.plan;
  long long leaf_cells = 0;
  for (long long c : p.tree_leaf_cells) leaf_cells += c;
  out8[0] = p.n_trees;
  out8[1] = p.dim;
  out8[2] = p.nc;
  out8[3] = p.min_lvl;
  out8[4] = p.max_lvl;
  out8[5] = p.n_slots;
  out8[6] = leaf_cells;
  out8[7] = f->f.bytes;
  return AFV_OK;
}

int afv_forest_set_var(afv_forest* f, int tree, int var, const double* host, int interior_only) {
  if (!f || !host) return fail(AFV_ERR_INVALID, "NULL argument");
  return guarded([&](std::string& err) -> int { return f->f.set_var(tree, var, host, interior_only, err); });
}

int afv_forest_get_var(afv_forest* f, int tree, int var, double* host, int interior_only) {
  if (!f || !host) return fail(AFV_ERR_INVALID, "NULL argument");
  return guarded([&](std::string& err) -> int { return f->f.get_var(tree, var, host, interior_only, err); });
}

int afv_forest_set_source(afv_forest* f, int tree, int src_lpl, int n_gauss, const double* gauss) {
  if (!f || (n_gauss > 0 && !gauss) || n_gauss < 0) return fail(AFV_ERR_INVALID, "bad arguments");
  return guarded([&](std::string& err) -> int {
    const afv::Plan& p = f->f.plan;
    if (tree < 0 || tree >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
    const int D = p.dim;
    std::vector<double> buf;
    for (int s : p.host_order[tree]) {
      int nc = p.nc_at(p.lvl[s]);
      int kmax = D == 3 ? nc : 1;
      for (int k = 1; k <= kmax; ++k)
        for (int j = 1; j <= nc; ++j)
          for (int i = 1; i <= nc; ++i) {
            int cix[3] = {i, j, k};
            double r[3];
            for (int d = 0; d < D; ++d) r[d] = p.r_min[(size_t)s * D + d] + (cix[d] - 0.5) * p.dr[s];
            buf.push_back(afv::source_eval(D, src_lpl, gauss, n_gauss, r));
          }
    }
    return f->f.set_var(tree, AFV_RHS, buf.data(), 1, err);
  });
}

int afv_forest_set_bc(afv_forest* f, int tree, int bc_type, int src_lpl, int n_gauss,
                      const double* gauss) {
  if (!f || (n_gauss > 0 && !gauss) || n_gauss < 0) return fail(AFV_ERR_INVALID, "bad arguments");
  if (bc_type != AFV_BC_DIRICHLET && bc_type != AFV_BC_NEUMANN)
    return fail(AFV_ERR_INVALID, "unknown boundary condition");
  return guarded([&](std::string& err) -> int {
    afv::Plan& p = f->f.plan;
    if (tree < 0 || tree >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
    afv::BcSpec& bc = p.bc[tree];
    bc.per_face = false;
    bc.face_type.clear();
    bc.face_vals.clear();
    bc.type = bc_type;
    bc.src_lpl = src_lpl;
    bc.gauss.assign(gauss ? gauss : nullptr, gauss ? gauss + (size_t)n_gauss * (2 + p.dim) : nullptr);
    afv::plan_fill_bc(p, tree);
    afv::plan_build_desc(p);
    return f->f.upload_bc(err);
  });
}

int afv_forest_set_bc_faces(afv_forest* f, int tree, long long n_faces, const int* bc_type,
                            long long n_values, const double* values) {
  if (!f || n_faces < 0 || n_values < 0 || (n_faces > 0 && !bc_type) || (n_values > 0 && !values))
    return fail(AFV_ERR_INVALID, "bad arguments");
  return guarded([&](std::string& err) -> int {
    afv::Plan& p = f->f.plan;
    if (tree < 0 || tree >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
    long long nf = 0, nv = 0;
    afv::plan_count_bc_faces(p, tree, nf, nv);
    if (nf != n_faces || nv != n_values)
      return err = "tree has " + std::to_string(nf) + " physical faces with " + std::to_string(nv) +
                   " face cells, got " + std::to_string(n_faces) + " and " + std::to_string(n_values),
             AFV_ERR_INVALID;
    for (long long i = 0; i < n_faces; ++i)
      if (bc_type[i] != AFV_BC_DIRICHLET && bc_type[i] != AFV_BC_NEUMANN)
        return err = "unknown boundary condition at face " + std::to_string(i), AFV_ERR_INVALID;
    afv::BcSpec& bc = p.bc[tree];
    bc.per_face = true;
    bc.gauss.clear();
    bc.face_type.assign(bc_type, bc_type + n_faces);
    bc.face_vals.assign(values, values + n_values);
    afv::plan_fill_bc(p, tree);
    afv::plan_build_desc(p);
    return f->f.upload_bc(err);
  });
}

int afv_forest_zero(afv_forest* f, int var) {
  if (!f) return fail(AFV_ERR_INVALID, "NULL argument");
  afv::Forest& F = f->f;
  cudaSetDevice(F.device);
  if (var == AFV_PHI) cudaMemsetAsync(F.d64.phi, 0, sizeof(double) * F.plan.n_elem_g, F.stream);
  else if (var == AFV_RHS) cudaMemsetAsync(F.d64.rhs, 0, sizeof(double) * F.plan.n_elem_i, F.stream);
  else if (var == AFV_TMP) cudaMemsetAsync(F.d64.tmp, 0, sizeof(double) * F.plan.n_elem_g, F.stream);
  else return fail(AFV_ERR_INVALID, "unknown variable");
  return AFV_OK;
}

int afv_forest_get_stream(afv_forest* f, void** stream) {
  if (!f || !stream) return fail(AFV_ERR_INVALID, "NULL argument");
  *stream = (void*)f->f.stream;
  return AFV_OK;
}

int afv_forest_sync(afv_forest* f) {
  if (!f) return fail(AFV_ERR_INVALID, "NULL argument");
  cudaSetDevice(f->f.device);
  cudaError_t e = cudaStreamSynchronize(f->f.stream);
  if (e != cudaSuccess) return fail(AFV_ERR_CUDA, cudaGetErrorString(e));
  return AFV_OK;
}

int afv_mg_init(afv_mg_opts* mg) {
  if (!mg) return fail(AFV_ERR_INVALID, "NULL argument");
  if (mg->n_cycle_down < 0) mg->n_cycle_down = 2;
  if (mg->n_cycle_up < 0) mg->n_cycle_up = 2;
  if (mg->n_cycle_base < 0) mg->n_cycle_base = 2;
  return AFV_OK;
}

#define FOREST_CALL(f, body)                                  \
  if (!(f)) return fail(AFV_ERR_INVALID, "forest is NULL");   \
  cudaSetDevice((f)->f.device);                               \
  return guarded([&](std::string& err) -> int { body; });

int afv_mg_fas_vcycle(afv_forest* f, const afv_mg_opts* mg, int highest_lvl, int set_residual) {
  FOREST_CALL(f, return f->f.vcycle(mg_of(mg), highest_lvl, set_residual != 0, err));
}

int afv_mg_fas_fmg(afv_forest* f, const afv_mg_opts* mg, int set_residual, int have_guess) {
  FOREST_CALL(f, return f->f.fmg(mg_of(mg), set_residual != 0, have_guess != 0, err));
}

int afv_gc_tree(afv_forest* f) { FOREST_CALL(f, return f->f.gc_tree(err)); }

int afv_forest_zero_tree(afv_forest* f, int tree, int var) {
  FOREST_CALL(f, return f->f.zero_tree(tree, var, err));
}


int afv_tree_max_abs_cc(afv_forest* f, int tree, int var, double* out) {
  if (!out) return fail(AFV_ERR_INVALID, "out is NULL");
  FOREST_CALL(f, return f->f.max_abs(tree, var, out, err));
}

int afv_tree_max_abs_cc_noalloc(afv_forest* f, int tree, int var, double* out) {
  if (!out) return fail(AFV_ERR_INVALID, "out is NULL");
  FOREST_CALL(f, return f->f.max_abs_static(tree, var, out, err));
}

int afv_mg_solve(afv_forest* f, const afv_mg_opts* mg, int precision, double tol, int max_cycles,
                 int* cycles, double* rel_res) {
  return afv_mg_solve_trees(f, mg, precision, tol, max_cycles, nullptr, cycles, rel_res);
}

int afv_mg_solve_trees(afv_forest* f, const afv_mg_opts* mg, int precision, double tol, int max_cycles,
                       const int* mask, int* cycles, double* rel_res) {
  if (precision != AFV_PREC_FP64 && precision != AFV_PREC_MIXED)
    return fail(AFV_ERR_INVALID, "unknown precision");
  if (!(tol > 0) || max_cycles < 0) return fail(AFV_ERR_INVALID, "bad tolerance or cycle limit");
  FOREST_CALL(f, {
    afv::SolveStats st;
    int rc = f->f.solve(mg_of(mg), precision, tol, max_cycles, st, err, mask);
    for (int t = 0; t < f->f.plan.n_trees; ++t) {
      if (cycles) cycles[t] = st.cycles.empty() ? 0 : st.cycles[t];
      if (rel_res) rel_res[t] = st.rel_res.empty() ? 0 : st.rel_res[t];
    }
    return rc;
  });
}

int afv_mg_gsrb_level(afv_forest* f, int lvl, int n_cycle) {
  FOREST_CALL(f, return f->f.gsrb_level(lvl, n_cycle, err));
}
int afv_fill_gc_level(afv_forest* f, int lvl) { FOREST_CALL(f, return f->f.fill_level(lvl, err)); }
int afv_mg_update_coarse(afv_forest* f, int lvl) {
  FOREST_CALL(f, return f->f.update_coarse(lvl, err));
}
int afv_mg_correct_children(afv_forest* f, int lvl_parent) {
  FOREST_CALL(f, return f->f.correct_children(lvl_parent, err));
}
int afv_mg_residual_all(afv_forest* f) { FOREST_CALL(f, return f->f.residual_all(nullptr, err)); }

int afv_forest_profile(afv_forest* f, int mask) {
  FOREST_CALL(f, {
    (void)err;
    f->f.prof_reset();
    f->f.prof_mask = mask;
    return AFV_OK;
  });
}

int afv_forest_profile_read(afv_forest* f, int kind, long long* launches, double* ms,
                            double* algorithmic_bytes) {
  if (!launches || !ms || !algorithmic_bytes) return fail(AFV_ERR_INVALID, "NULL argument");
  if (kind == -1) {
    if (!f) return fail(AFV_ERR_INVALID, "forest is NULL");
    *launches = f->f.n_launches;
    *ms = 0;
    *algorithmic_bytes = 0;
    return AFV_OK;
  }
  if (kind < 0 || kind >= afv::kProfKinds) return fail(AFV_ERR_INVALID, "unknown kernel kind");
  FOREST_CALL(f, {
    (void)err;
    return f->f.prof_read(kind, launches, ms, algorithmic_bytes);
  });
}

int afv_forest_profile_entries(afv_forest* f, long long max, int* kind, int* level, double* ms,
                               double* algorithmic_bytes, int* launches, long long* n_total) {
  if (!n_total || (max > 0 && (!kind || !level || !ms || !algorithmic_bytes || !launches)))
    return fail(AFV_ERR_INVALID, "NULL argument");
  FOREST_CALL(f, {
    (void)err;
    *n_total = f->f.prof_entries(max, kind, level, ms, algorithmic_bytes, launches);
    return AFV_OK;
  });
}

int afv_forest_set_option(afv_forest* f, int option, int value) {
  if (!f) return fail(AFV_ERR_INVALID, "forest is NULL");
  switch (option) {
    case AFV_OPT_SWEEP_KERNEL:
      if (value < 0 || value > 5) return fail(AFV_ERR_INVALID, "sweep kernel must be 0 .. 5");
      f->f.sweep_kernel = value;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_GRAPHS:
      f->f.use_graphs = value != 0;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_RESTRICT_KERNEL:
      if (value != 0 && value != 1) return fail(AFV_ERR_INVALID, "restrict kernel must be 0 or 1");
      f->f.use_restrict_warp = value != 0;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_SMALL_SWEEPS:
      f->f.use_small_sweeps = value != 0;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_PROFILE_LEAD_US:
      if (value < 0 || value > 1000000) return fail(AFV_ERR_INVALID, "profile lead must be 0 .. 1e6 us");
      f->f.prof_lead_us = value;
      return AFV_OK;
    case AFV_OPT_DEFECT_KERNEL:
      if (value != 0 && value != 1) return fail(AFV_ERR_INVALID, "defect kernel must be 0 or 1");
      f->f.defect_fx = value != 0;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_DEFECT_CELLS:
      if (value != 0 && value != 1 && value != 2 && value != 4)
        return fail(AFV_ERR_INVALID, "defect cells per thread must be 0, 1, 2 or 4");
      f->f.defect_cells = value;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_COARSE_END:
      f->f.use_coarse_end = value != 0;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_ZERO_COPY:
      f->f.zero_copy = value != 0;
      return AFV_OK;
    case AFV_OPT_DIRECT_BOXES:
      if (value < -1) return fail(AFV_ERR_INVALID, "direct boxes must be >= -1");
      f->f.direct_boxes = value;
      f->f.drop_graphs();
      return AFV_OK;
    case AFV_OPT_WAIT_LIMIT_US:
      if (value < 0) return fail(AFV_ERR_INVALID, "wait limit must be >= 0 us");
      // clock64() counts SM cycles: about 2000 per microsecond at GB300 clocks
      f->f.meta.wait_limit = 2000LL * value;
      f->f.drop_graphs();  // captured launches hold the old limit
      return AFV_OK;
  }
  return fail(AFV_ERR_INVALID, "unknown option");
}

int afv_forest_get_option(afv_forest* f, int option, int* value) {
  if (!f || !value) return fail(AFV_ERR_INVALID, "NULL argument");
  switch (option) {
    case AFV_OPT_SWEEP_KERNEL: *value = f->f.sweep_kernel; return AFV_OK;
    case AFV_OPT_GRAPHS: *value = f->f.use_graphs ? 1 : 0; return AFV_OK;
    case AFV_OPT_RESTRICT_KERNEL: *value = f->f.use_restrict_warp ? 1 : 0; return AFV_OK;
    case AFV_OPT_SMALL_SWEEPS: *value = f->f.use_small_sweeps ? 1 : 0; return AFV_OK;
    case AFV_OPT_PROFILE_LEAD_US: *value = f->f.prof_lead_us; return AFV_OK;
    case AFV_OPT_DEFECT_KERNEL: *value = f->f.defect_fx ? 1 : 0; return AFV_OK;
    case AFV_OPT_DEFECT_CELLS: *value = f->f.defect_cells; return AFV_OK;
    case AFV_OPT_COARSE_END: *value = f->f.use_coarse_end ? 1 : 0; return AFV_OK;
    case AFV_OPT_WAIT_LIMIT_US: *value = (int)(f->f.meta.wait_limit / 2000LL); return AFV_OK;
    case AFV_OPT_DIRECT_BOXES: *value = f->f.direct_boxes; return AFV_OK;
    case AFV_OPT_ZERO_COPY: *value = f->f.zero_copy ? 1 : 0; return AFV_OK;
  }
  return fail(AFV_ERR_INVALID, "unknown option");
}

int afv_mg_set_operator(afv_forest* f, int op, int i_eps) { return afv_mg_set_operator_lsf(f, op, i_eps, -1, -1); }

int afv_mg_set_operator_lsf(afv_forest* f, int op, int i_eps, int i_lsf, int i_bval) {
  FOREST_CALL(f, return f->f.set_operator(op, i_eps, i_lsf, i_bval, err));
}

int afv_forest_add_vars(afv_forest* f, int n_cc, int n_fc) {
  FOREST_CALL(f, return afv::forest_add_vars(f->f, n_cc, n_fc, err));
}

static int fc_exchange(afv_forest* f, int tree, int ifc, double* host, long long n, bool to_dev) {
  if (!f || !host) return fail(AFV_ERR_INVALID, "NULL argument");
  cudaSetDevice(f->f.device);
  return guarded([&](std::string& err) -> int {
    if (tree < 0 || tree >= f->f.plan.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
    if (n != afv::forest_fc_count(f->f, tree)) return err = "value count does not match the tree", AFV_ERR_INVALID;
    return afv::forest_fc_exchange(f->f, tree, ifc, host, to_dev, err);
  });
}

int afv_forest_set_fc(afv_forest* f, int tree, int ifc, const double* host, long long n) {
  return fc_exchange(f, tree, ifc, const_cast<double*>(host), n, true);
}

int afv_forest_get_fc(afv_forest* f, int tree, int ifc, double* host, long long n) {
  return fc_exchange(f, tree, ifc, host, n, false);
}

int afv_prolong_from_level(afv_forest* f, int lvl_parent, int iv, int iv_to, int order, int add) {
  FOREST_CALL(f, return afv::forest_prolong(f->f, lvl_parent, iv, iv_to, order, add, err));
}

int afv_restrict_tree(afv_forest* f, int iv, int iv_to) {
  FOREST_CALL(f, return afv::forest_restrict_tree(f->f, iv, iv_to, err));
}

int afv_gc_tree_var(afv_forest* f, int iv, int rb_method, int bc_method) {
  FOREST_CALL(f, return afv::forest_gc_tree_var(f->f, iv, rb_method, bc_method, err));
}

int afv_gc2_level(afv_forest* f, int tree, int lvl, int iv, double* host_out, long long n_out) {
  if (!host_out) return fail(AFV_ERR_INVALID, "NULL argument");
  FOREST_CALL(f, return afv::forest_gc2_level(f->f, tree, lvl, iv, host_out, n_out, err));
}

int afv_consistent_fluxes(afv_forest* f, int n_fc, const int* f_ixs) {
  FOREST_CALL(f, return afv::forest_consistent_fluxes(f->f, n_fc, f_ixs, err));
}

int afv_write_vtk(afv_forest* f, int tree, const char* filename, int n_cycle, double time, int n_cc,
                  const int* ixs_cc, const char* const* cc_names, int n_fc, const int* ixs_fc,
                  const char* const* fc_names, const char* dir) {
  FOREST_CALL(f, return afv::forest_write_vtk(f->f, tree, filename, n_cycle, time, n_cc, ixs_cc, cc_names, n_fc,
                                              ixs_fc, fc_names, dir, err));
}

int afv_forest_autotune(afv_forest* f, int* choice, float* ms3) {
  FOREST_CALL(f, return f->f.autotune(choice, ms3, err));
}

int afv_forest_autotune_all(afv_forest* f, int* choice3, float* ms10) {
  if (!choice3) return fail(AFV_ERR_INVALID, "NULL argument");
  FOREST_CALL(f, return f->f.autotune_all(&choice3[0], &choice3[1], &choice3[2], ms10, err));
}

int afv_forest_autotune_defect(afv_forest* f, int* cells, float* ms3) {
  FOREST_CALL(f, return f->f.autotune_defect(cells, ms3, err));
}

int afv_forest_set_source_device(afv_forest* f, int tree, int src_lpl, int n_gauss, const double* gauss) {
  if (n_gauss < 0 || (n_gauss > 0 && !gauss)) return fail(AFV_ERR_INVALID, "bad arguments");
  FOREST_CALL(f, return f->f.set_source_device(tree, src_lpl, n_gauss, gauss, err));
}

}  // extern "C"
