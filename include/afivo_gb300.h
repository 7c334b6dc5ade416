/*
 * afivo_gb300 — C ABI of a GB300 (sm_103a) FAS multigrid solver for Poisson
 * problems on quadtree/octree block grids.
 *
 * Every entry point here replaces one routine of the Afivo reference's Fortran
 * API for this path; the citation beside each names it (file:line, paths
 * relative to the reference project). fortran/m_afivo_gb300.f90 binds these
 * functions through iso_c_binding, and fortran/m_aX_gb300.f90 (expanded to
 * modules m_a2_gb300 / m_a3_gb300) provides mg2_fas_vcycle, mg2_fas_fmg,
 * mg3_fas_vcycle and mg3_fas_fmg with the reference's names and arguments
 * on the reference's own tree type.
 *
 * Conventions
 *  - Every function returns AFV_OK (0) or a negative AFV_ERR_* code; it never
 *    aborts the process (the reference calls `stop`). afv_last_error() gives
 *    the message of the calling thread's last failure.
 *  - Box ids, levels, ix indices and neighbour codes follow the reference:
 *    ids are 1-based, ix is 1-based, a neighbour id > 0 is a box, 0 means no
 *    box (refinement boundary) and < 0 a physical boundary
 *    (src/m_aX_t.f90:32-33, src/m_aX_gc.f90:58-67).
 *  - Host cell data is exchanged as the reference stores it: per box an array
 *    cc(0:nc+1, 0:nc+1[, 0:nc+1]) with x fastest, boxes in the order of the
 *    tree's level lists (lvls(min_lvl)%ids, ..., lvls(highest_lvl)%ids).
 *  - Device calls are ordered on the forest's CUDA stream. Calls on one
 *    forest are not re-entrant (like the reference's routines on one tree).
 */
#ifndef AFIVO_GB300_H
#define AFIVO_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  AFV_OK = 0,
  AFV_ERR_INVALID = -1,     /* bad argument or malformed tree            */
  AFV_ERR_CUDA = -2,        /* a CUDA runtime call failed                */
  AFV_ERR_NOMEM = -3,       /* host or device allocation failed          */
  AFV_ERR_UNSUPPORTED = -4, /* valid request this build does not support */
  AFV_ERR_TIMEOUT = -5,     /* a bounded device wait gave up (the device
                               error word was set; it is cleared on report) */
  AFV_ERR_STATE = -6,       /* call out of order (e.g. before set_base)  */
  AFV_ERR_BUDGET = -7,      /* over the memory budget (box_limit, HBM)   */
  AFV_ERR_DIVERGED = -8,    /* a solve produced a non-finite residual    */
  AFV_ERR_NOT_CONVERGED = -9 /* a solve ran max_cycles without reaching tol */
};

/* Refinement flags, src/m_aX_t.f90:17-24. */
enum { AFV_RM_REF = -1, AFV_KEEP_REF = 0, AFV_DO_REF = 1 };

/* Cell-centred variables of a forest (mg%i_phi, mg%i_rhs, mg%i_tmp). */
enum { AFV_PHI = 0, AFV_RHS = 1, AFV_TMP = 2 };

/* Boundary-condition types, src/m_aX_t.f90:45-49. */
enum { AFV_BC_DIRICHLET = -1, AFV_BC_NEUMANN = -2 };

/* Built-in refinement criteria (afv_ref_crit.kind). */
enum {
  AFV_REF_UNIFORM = 0,  /* do_ref while lvl < lvl_max                        */
  AFV_REF_SOURCE = 1,   /* do_ref if any cell centre has |f|*dr^2 > thr      */
  AFV_REF_RANDOM = 2,   /* do_ref with probability prob (keyed, seeded)      */
  AFV_REF_RANDOM_RM = 3 /* as RANDOM, and rm_ref otherwise                   */
};

/* Solver precisions (afv_mg_solve). */
enum { AFV_PREC_FP64 = 0, AFV_PREC_MIXED = 1 };

typedef struct afv_tree afv_tree;     /* host tree, the reference's a$D_t   */
typedef struct afv_forest afv_forest; /* device-resident set of trees       */

/* What a refinement callback sees of a box (box$D_t, src/m_aX_t.f90:153-177). */
typedef struct {
  int id, lvl, n_cell, dim;
  int ix[3];
  double dr;
  double r_min[3];
  int pass; /* number of adjust_refinement calls made before this one */
} afv_box_view;

/* The reference's ref_subr hook, src/m_aX_t.f90:231-236. */
typedef void (*afv_ref_fn)(const afv_box_view* box, int* ref_flag, void* user);

/* Parameters of a built-in criterion. Sources are sums of Gaussians
 * a*exp(-|r-c|^2/s^2) (src_lpl = 0) or their Laplacian (src_lpl = 1), in the
 * form of examples/m_gaussians.f90:64-102; gauss holds n_gauss records of
 * (a, s, c_1..c_dim). */
typedef struct {
  int kind;
  int lvl_max;
  double thr;
  double prob;
  unsigned long long seed;
  int src_lpl;
  int n_gauss;
  const double* gauss;
} afv_ref_crit;

/* Multigrid options, the mg$D_t type of src/m_aX_mg.f90:20-52. Negative cycle
 * counts mean the reference defaults (2), src/m_aX_mg.f90:142-144. */
typedef struct {
  int n_cycle_down;
  int n_cycle_up;
  int n_cycle_base;
} afv_mg_opts;

typedef struct {
  int device;         /* CUDA device ordinal                                 */
  int mixed_buffers;  /* 1: also allocate the FP32 state for AFV_PREC_MIXED  */
} afv_forest_opts;

/* ---- errors -------------------------------------------------------------- */
const char* afv_last_error(void);
int afv_version(void);

/* ---- tree build (host) --------------------------------------------------- */

/* a$D_init, src/m_aX_core.f90:24-131 (n_var_cell is fixed to phi, rhs, tmp;
 * coarsen_to <= 0 means no coarse sub-levels). */
int afv_tree_create(int dim, int n_cell, double dr, const double* r_min, int lvl_limit,
                    int coarsen_to, double mem_limit_gb, afv_tree** out);
/* a$D_init's coord argument (src/m_aX_core.f90:58-70, 102): AFV_COORD_CYL
 * makes a 2-D tree cylindrical (x the radius, y the axis). Set it before
 * afv_tree_set_base; every box inherits it (core:772). */
enum { AFV_COORD_XYZ = 0, AFV_COORD_CYL = 1 };
int afv_tree_set_coord(afv_tree* t, int coord);
/* a$D_set_base, src/m_aX_core.f90:152-235. ix_list: n_boxes*dim, nb_list:
 * n_boxes*2*dim, both box-major. */
int afv_tree_set_base(afv_tree* t, int n_boxes, const int* ix_list, const int* nb_list);
/* a$D_adjust_refinement, src/m_aX_core.f90:452-541 (one pass, at most one
 * level per call); n_add / n_rm are ref_info%n_add / ref_info%n_rm. */
int afv_tree_adjust_refinement(afv_tree* t, afv_ref_fn fn, void* user, int* n_add, int* n_rm);
/* a$D_adjust_refinement with a built-in criterion. */
int afv_tree_adjust_builtin(afv_tree* t, const afv_ref_crit* crit, int* n_add, int* n_rm);
/* The examples' "do; adjust_refinement; if (n_add == 0) exit" loop
 * (examples/poisson_basic_2d.f90:59-68). */
int afv_tree_refine_builtin(afv_tree* t, const afv_ref_crit* crit, int max_passes,
                            int* n_passes);
/* a$D_destroy, src/m_aX_core.f90:135-148. */
void afv_tree_destroy(afv_tree* t);
/* out[8] = dim, n_cell, min_lvl, highest_lvl, highest_id, boxes in use,
 * leaves, lvl_limit (a$D_print_info, src/m_aX_t.f90:303-329). */
int afv_tree_get_info(const afv_tree* t, int* out8);
/* Per-id topology (rows id-1, ids 1..highest_id) of box$D_t. */
int afv_tree_export(const afv_tree* t, int* lvl, int* ix, int* parent, int* children,
                    int* neighbors, int* n_cell, double* dr, double* r_min, int* in_use);
/* lvls(lvl)%ids / %leaves / %parents (lvl_t, src/m_aX_t.f90:181-185);
 * sizes3 receives the three lengths; the list pointers may be NULL. */
int afv_tree_level(const afv_tree* t, int lvl, int* sizes3, int* ids, int* leaves, int* parents);

/* ---- tree build on the device ------------------------------------------------ */

typedef struct afv_dtree afv_dtree; /* a tree held and refined in device memory */

/* No counterpart in the reference (its tree lives in host memory): a device
 * copy of a host tree (after a$D_set_base or any refinement), for refining
 * without moving the tree through host memory. */
int afv_dtree_create(const afv_tree* t, int device, afv_dtree** out);
void afv_dtree_destroy(afv_dtree* t);
/* a$D_adjust_refinement on the device (src/m_aX_core.f90:452-541, with
 * consistent_ref_flags :628-725, add_children / remove_children :728-787,
 * set_neighbs :387-422 and a$D_tidy_up :238-314), for a built-in criterion
 * (at most 16 Gaussians): the same ids, links and level lists as
 * afv_tree_adjust_builtin on the host. Only list sizes and counts come back
 * to the host during a pass. */
int afv_dtree_adjust_builtin(afv_dtree* t, const afv_ref_crit* crit, int* n_add, int* n_rm);
/* afv_tree_refine_builtin's loop with afv_dtree_adjust_builtin. */
int afv_dtree_refine_builtin(afv_dtree* t, const afv_ref_crit* crit, int max_passes, int* n_passes);
/* Replaces the state of host tree `host` by the device tree's (for instance
 * to create a forest from it). */
int afv_dtree_download(const afv_dtree* t, afv_tree* host);
/* out[5] = highest_lvl, highest_id, adjust passes made, boxes in use, leaves. */
int afv_dtree_get_info(const afv_dtree* t, int* out5);

/* ---- device forest ----------------------------------------------------------- */

/* Uploads the topology of n_trees trees (same dim, n_cell, coarsen_to) and
 * allocates their cell data on the device, zero-initialised. One forest is
 * swept by one kernel launch per level and operator. */
int afv_forest_create(int n_trees, afv_tree* const* trees, const afv_forest_opts* opts,
                      afv_forest** out);
void afv_forest_destroy(afv_forest* f);
/* out[8] = n_trees, dim, n_cell, min_lvl, max_lvl, boxes, leaf cells, device bytes. */
int afv_forest_get_info(const afv_forest* f, long long* out8);
/* Copy one variable of one tree to or from the host, in the reference's box
 * layout (see conventions). interior_only = 1 packs only cc(1:nc,...) per box. */
int afv_forest_set_var(afv_forest* f, int tree, int var, const double* host, int interior_only);
int afv_forest_get_var(afv_forest* f, int tree, int var, double* host, int interior_only);
/* Fill rhs of one tree with a Gaussian source at the cell centres. */
int afv_forest_set_source(afv_forest* f, int tree, int src_lpl, int n_gauss, const double* gauss);
/* afv_forest_set_source evaluated on the device (at most 16 Gaussians), for
 * callers that stream many trees (a request loop): microseconds instead of
 * the host evaluation's seconds for a 256^3 tree. Uses the device's exp, so
 * values may differ from the host evaluation in the last bit. */
int afv_forest_set_source_device(afv_forest* f, int tree, int src_lpl, int n_gauss,
                                 const double* gauss);
/* Boundary values on physical faces of one tree: the sides_bc hook of the
 * reference (src/m_aX_t.f90:276-282) sampled once. bc_type is AFV_BC_*; the
 * boundary value is 0 when n_gauss == 0, else the Gaussian source at the face
 * centres (examples/poisson_basic_2d.f90:167-203). */
int afv_forest_set_bc(afv_forest* f, int tree, int bc_type, int src_lpl, int n_gauss,
                      const double* gauss);
/* The sides_bc hook of the reference (src/m_aX_t.f90:276-282), sampled on
 * the host for every physical-boundary face of one tree: bc_type[i] (AFV_BC_*)
 * and nc^(D-1) boundary values per face, in the order of the ghost cells
 * cc(0, 1:nc[, 1:nc]) etc. (first tangential index fastest). Faces are listed
 * box by box in the host exchange order, faces of a box low x, high x, low y,
 * ... and only those whose neighbour is < 0. n_faces and n_values must match
 * the tree. Used by bc_to_gc (src/m_aX_gc.f90:71-132) as the reference uses
 * the hook's output. */
int afv_forest_set_bc_faces(afv_forest* f, int tree, long long n_faces, const int* bc_type,
                            long long n_values, const double* values);
int afv_forest_zero(afv_forest* f, int var);
/* No counterpart in the reference: a$D_box_clear_cc (src/m_aX_utils.f90:
 * 262-270) on every box of one tree of the forest. */
int afv_forest_zero_tree(afv_forest* f, int tree, int var);
int afv_forest_sync(afv_forest* f);
/* No counterpart in the reference: the cudaStream_t that orders this
 * forest's work, for callers that time it or order their own work after it. */
int afv_forest_get_stream(afv_forest* f, void** stream);

/* ---- multigrid ------------------------------------------------------------------- */

/* mg$D_init_mg, src/m_aX_mg.f90:130-154. */
int afv_mg_init(afv_mg_opts* mg);
/* Operators of the multigrid routines (mg%box_op, mg%box_gsrb, mg%box_corr,
 * mg%box_rstr): AFV_OP_LPL, the constant-coefficient Laplacian
 * (mg$D_box_*_lpl, the default); AFV_OP_LPLD, the variable-coefficient
 * operator div(eps grad phi) on every box (mg$D_box_gsrb_lpld, mg$D_box_lpld,
 * mg$D_box_corr_lpld, src/m_aX_mg.f90:810-985); AFV_OP_CLPL / AFV_OP_CLPLD,
 * their cylindrical forms (mg2_box_*_clpl, mg2_box_*_clpld, :1323-1443;
 * cylindrical 2-D trees only); AFV_OP_LPLLSF, the Laplacian with internal
 * boundaries where a level set changes sign (mg$D_box_*_lpllsf with
 * mg$D_box_rstr_lpllsf, :987-1321); AFV_OP_AUTO, the per-box dispatch of
 * mg$D_auto_gsrb / _op / _corr / _rstr (:562-669) by the tags of
 * mg$D_set_box_tag. In cylindrical trees every operator restricts with the
 * radial weights of a2_restrict_box (src/m_aX_restrict.f90:90-103). */
enum { AFV_OP_LPL = 0, AFV_OP_LPLD = 1, AFV_OP_AUTO = 2, AFV_OP_CLPL = 3, AFV_OP_CLPLD = 4, AFV_OP_LPLLSF = 5 };
/* Sets mg%box_op / box_gsrb / box_corr / box_rstr and mg%i_eps of a forest
 * (mg%i_lsf = mg%i_bval = -1). eps is the extra cell variable i_eps (>= 3,
 * afv_forest_add_vars); as with the reference, the caller fills its ghost
 * cells and coarse levels (for instance afv_gc_tree_var and
 * afv_restrict_tree). For AFV_OP_AUTO the per-box tags of mg$D_set_box_tag
 * (:672-706, min and max of eps and of the level set over the box, ghost
 * cells included) are taken by this call, where the reference takes each
 * box's tag at its first use: call it again after changing eps or the level
 * set. A box that would take two tags is refused with AFV_ERR_INVALID, where
 * the reference stops. The operator applies to the FP64 routines (V-cycle,
 * FMG, single operators, FP64 solves); a mixed-precision solve with another
 * operator than the Cartesian Laplacian returns AFV_ERR_UNSUPPORTED. */
int afv_mg_set_operator(afv_forest* f, int op, int i_eps);
/* As afv_mg_set_operator, with mg%i_lsf and mg%i_bval (both >= 3 or both
 * -1, mg$D_init_mg's check, src/m_aX_mg.f90:136-137): the level set and the
 * boundary value at the interface, extra cell variables with filled ghost
 * cells. AFV_OP_LPLLSF needs both; AFV_OP_AUTO without eps or a level set
 * tags every box normal (examples/poisson_cyl.f90). */
int afv_mg_set_operator_lsf(afv_forest* f, int op, int i_eps, int i_lsf, int i_bval);
/* mg$D_fas_vcycle, src/m_aX_mg.f90:208-255 (all trees of the forest). */
int afv_mg_fas_vcycle(afv_forest* f, const afv_mg_opts* mg, int highest_lvl, int set_residual);
/* mg$D_fas_fmg, src/m_aX_mg.f90:164-203. */
int afv_mg_fas_fmg(afv_forest* f, const afv_mg_opts* mg, int set_residual, int have_guess);
/* a$D_gc_tree(tree, i_phi, mg%sides_rb, mg%sides_bc), src/m_aX_gc.f90:28-46. */
int afv_gc_tree(afv_forest* f);
/* max(|a$D_tree_min_cc|, |a$D_tree_max_cc|) over leaf interiors,
 * src/m_aX_utils.f90:468-571. */
int afv_tree_max_abs_cc(afv_forest* f, int tree, int var, double* out);
/* afv_tree_max_abs_cc without any allocation (no counterpart in the
 * reference): the reduction scratch is a static device array of 536,576
 * bytes per device, which limits it to forests of at most 1024 trees
 * (larger ones get AFV_ERR_INVALID). The first call on a device takes the
 * array's address (cudaGetSymbolAddress) and should come before any stream
 * capture; so does the first call after a device reset, which takes it
 * again. Every call clears the scratch it uses on the forest's stream.
 * Calls that overlap in time on one device (two host threads, or two forests
 * on different streams) share the scratch and race: serialise them. For
 * callers that cannot allocate at the time of the call: a request loop whose
 * device memory is fully committed to admitted trees, where an allocation
 * would fail, and loops that poll a norm often, where every cudaMalloc and
 * cudaFree would synchronise the device. */
int afv_tree_max_abs_cc_noalloc(afv_forest* f, int tree, int var, double* out);
/* Solve every tree to max|rhs - L phi| <= tol * max|rhs| over its leaves,
 * from the current phi, with FP64 V-cycles (AFV_PREC_FP64) or FP64 defect
 * correction around FP32 V-cycles (AFV_PREC_MIXED). cycles[t] and rel_res[t]
 * (n_trees entries, may be NULL) receive per-tree results. Returns
 * AFV_ERR_NOT_CONVERGED if a tree is not converged after max_cycles,
 * AFV_ERR_DIVERGED if a tree's residual stopped being finite, and
 * AFV_ERR_TIMEOUT if a bounded device wait gave up during the solve. */
int afv_mg_solve(afv_forest* f, const afv_mg_opts* mg, int precision, double tol, int max_cycles,
                 int* cycles, double* rel_res);
/* No counterpart in the reference: afv_mg_solve on the trees whose mask
 * entry is nonzero (mask may be NULL: every tree); the other trees' cell
 * data is left as it is and their cycles / rel_res entries are 0. A forest
 * whose trees are request slots solves the occupied slots only; when those
 * are the leading slots (mask 1..1 0..0) the launches cover only their boxes,
 * so the cost follows the number of occupied slots. */
int afv_mg_solve_trees(afv_forest* f, const afv_mg_opts* mg, int precision, double tol, int max_cycles,
                       const int* mask, int* cycles, double* rel_res);

/* Single operators of the V-cycle, one level of every tree. */
/* gsrb_boxes, src/m_aX_mg.f90:397-420 */
int afv_mg_gsrb_level(afv_forest* f, int lvl, int n_cycle);
/* fill_gc_phi, src/m_aX_mg.f90:352-365 */
int afv_fill_gc_level(afv_forest* f, int lvl);
/* update_coarse, src/m_aX_mg.f90:424-480 */
int afv_mg_update_coarse(afv_forest* f, int lvl);
/* correct_children, src/m_aX_mg.f90:368-395 (parents at lvl_parent) */
int afv_mg_correct_children(afv_forest* f, int lvl_parent);
/* residual_box on every box of every level, src/m_aX_mg.f90:243-254 */
int afv_mg_residual_all(afv_forest* f);

/* ---- general ghost cells, transfers and output ------------------------------ */

/* Refinement-boundary methods of afv_gc_tree_var (the reference's sides_rb
 * hooks): mg$D_sides_rb (src/m_aX_mg.f90:262-350), a$D_gc_prolong0
 * (src/m_aX_gc.f90:135-151), a$D_gc_interp (:155-245) and a$D_gc_interp_lim
 * (:249-358). */
enum { AFV_RB_MG = 0, AFV_RB_PROLONG0 = 1, AFV_RB_INTERP = 2, AFV_RB_INTERP_LIM = 3 };
/* Physical-boundary methods of afv_gc_tree_var: the forest's sampled sides_bc
 * records (afv_forest_set_bc / _set_bc_faces), or a$D_bc_dirichlet_zero /
 * a$D_bc_neumann_zero (src/m_aX_gc.f90:361-378). */
enum { AFV_BCM_TABLE = 0, AFV_BCM_DIRICHLET_ZERO = -1, AFV_BCM_NEUMANN_ZERO = -2 };

/* The n_var_cell / n_var_face arguments of a$D_init (src/m_aX_core.f90:24-50)
 * for a forest: adds n_cc cell-centred FP64 variables (numbered 3, 4, ...,
 * ghosted like phi, exchanged with afv_forest_set_var / _get_var) and n_fc
 * face variables (fx, fy[, fz] of box$D_t, src/m_aX_t.f90:153-177),
 * zero-initialised. Face variables can be added once. */
int afv_forest_add_vars(afv_forest* f, int n_cc, int n_fc);
/* Face variable ifc of one tree to or from the host: per box in the host
 * exchange order, fx(1:nc+1,1:nc[,1:nc]), then fy, then fz, x fastest;
 * n = the total count (checked). */
int afv_forest_set_fc(afv_forest* f, int tree, int ifc, const double* host, long long n);
int afv_forest_get_fc(afv_forest* f, int tree, int ifc, double* host, long long n);
/* a$D_prolong0_from / a$D_prolong1_from / a$D_prolong2_from
 * (src/m_aX_prolong.f90:22-37, 112-127, 226-241) for order 0 / 1 / 2 on every
 * parent of level lvl_parent of every tree: cell variable iv of the parents
 * into iv_to of their children, added to the old values when add != 0. The
 * parents' ghost cells must be valid for orders 1 and 2. */
int afv_prolong_from_level(afv_forest* f, int lvl_parent, int iv, int iv_to, int order, int add);
/* a$D_restrict_tree, src/m_aX_restrict.f90:54-64 (iv into iv_to on every
 * parent, finest level first). */
int afv_restrict_tree(afv_forest* f, int iv, int iv_to);
/* a$D_gc_tree(tree, iv, subr_rb, subr_bc), src/m_aX_gc.f90:28-46, with
 * subr_rb one of AFV_RB_* and subr_bc one of AFV_BCM_*, for a ghosted cell
 * variable iv. */
int afv_gc_tree_var(afv_forest* f, int iv, int rb_method, int bc_method);
/* a$D_gc2_box (src/m_aX_gc.f90:420-440) with subr_rb = a$D_gc2_prolong1 and
 * subr_bc = a$D_bc2_neumann_zero, for every box of one tree on level lvl
 * (>= 1), in level-list order: host_out receives per box gc_data(nc[,nc],
 * 2D), the second layer of ghost cells per face. n_out must be boxes x 2D x
 * nc^(D-1). */
int afv_gc2_level(afv_forest* f, int tree, int lvl, int iv, double* host_out, long long n_out);
/* a$D_consistent_fluxes, src/m_aX_core.f90:811-945 (Cartesian): face
 * variables f_ixs[0..n_fc-1] of leaves next to refined neighbours become the
 * averages of the neighbours' fine fluxes. */
int afv_consistent_fluxes(afv_forest* f, int n_fc, const int* f_ixs);
/* a$D_write_vtk, src/m_aX_io.f90:115-310: the leaves of levels 1..highest of
 * one tree as a VTK unstructured grid, file filename.vtu (in dir, if given),
 * with the cell variables ixs_cc (names cc_names) and the cell averages of
 * the face variables ixs_fc (names fc_names + "_x", "_y"[, "_z"]). The file
 * layout is that of src/m_vtk.f90 (appended raw data); the TIME and CYCLE
 * values are written as %.17E and %d text. */
int afv_write_vtk(afv_forest* f, int tree, const char* filename, int n_cycle, double time, int n_cc,
                  const int* ixs_cc, const char* const* cc_names, int n_fc, const int* ixs_fc,
                  const char* const* fc_names, const char* dir);

/* ---- measurement ------------------------------------------------------------ */

/* Kernel kinds of the event profiler. */
enum {
  AFV_KERNEL_SWEEP = 0,     /* GSRB half-sweep (with the pulled ghost fill)  */
  AFV_KERNEL_FILL = 1,      /* ghost fill of a level                         */
  AFV_KERNEL_RESTRICT = 2,  /* residual + restriction to the parents         */
  AFV_KERNEL_COARSE_RHS = 3,
  AFV_KERNEL_CORRECT = 4,   /* coarse correction with prolong2               */
  AFV_KERNEL_RESIDUAL = 5,
  AFV_KERNEL_DEFECT = 6,    /* FP64 defect of the mixed path                 */
  AFV_KERNEL_ACCUMULATE = 7, /* FP64 accumulate of the FP32 correction       */
  AFV_KERNEL_COARSE_END = 8  /* correction cycle's levels <= 1, one launch    */
};
/* No counterpart in the reference (it has no GPU path): bracket every launch
 * of the kinds in mask (bit k = kind k) with CUDA events on the forest's
 * stream; mask = 0 switches it off and drops the records. */
int afv_forest_profile(afv_forest* f, int mask);
/* Launch count, summed event time (ms) and summed algorithmic bytes of the
 * launches of one kind since profiling was switched on. kind = -1 gives the
 * number of kernels launched on the forest's stream since it was created. */
int afv_forest_profile_read(afv_forest* f, int kind, long long* launches, double* ms,
                            double* algorithmic_bytes);
/* No counterpart in the reference: tuning switches of a forest (the
 * autotuner sets them). AFV_OPT_SWEEP_KERNEL: 0 block-pipelined level kernel,
 * 1 warp-per-box kernel with bulk copies (default), 2 warp-per-box kernel with
 * per-lane asynchronous copies. AFV_OPT_GRAPHS: 1 (default) runs each solve as
 * one CUDA graph (its iterations repeated on the device), 0 launches the
 * kernels one by one with the host deciding every iteration.
 * AFV_OPT_RESTRICT_KERNEL: 1 (default) warp-per-box kernels for the residual
 * restriction (levels >= 2), the coarse right-hand side (levels >= 1) and the
 * correction of children on levels >= 2, 0 the block-staged kernels. AFV_OPT_SMALL_SWEEPS: 1 (default) runs all
 * half-sweeps of a level of at most 2048 interior cells in one block, 0
 * launches them one by one. AFV_OPT_PROFILE_LEAD_US: with the event profiler
 * on, each solve iteration is queued behind a device-side wait of this many
 * microseconds (default 0), so that the events time the kernels rather than
 * the host's launch rate. AFV_OPT_DEFECT_KERNEL: the mixed solve's FP64
 * defect r = f - L u computes the Laplacian in 64-bit fixed point per box
 * (1, default; exact sums, one FP64 multiply-add per cell) or as an FP64 sum
 * (0). AFV_OPT_SWEEP_KERNEL 3..5 are other warp and stage counts of 1.
 * AFV_OPT_COARSE_END: 1 (default) runs the mixed solve's correction cycle on
 * levels <= 1 (one box per tree each) in one launch, one block per tree;
 * 0 launches its operators one by one. AFV_OPT_WAIT_LIMIT_US: how long
 * (microseconds, default 2000000) a kernel waits for one of its own copies
 * into shared memory before it gives up, sets the device error word and
 * returns once its copies in flight have landed; the call then reports
 * AFV_ERR_TIMEOUT and clears the word. 0 makes every such wait give up at
 * once, which exercises that path without a stuck copy.
 * AFV_OPT_DIRECT_BOXES: levels of at most this many boxes (0: none) take the
 * unstaged half-sweep, one thread per updated cell reading its neighbours
 * and pulled ghosts straight from memory (same values); -1 (default): FP64
 * sweeps on every level, FP32 sweeps never. AFV_OPT_ZERO_COPY: 1 (default)
 * exchanges page-locked host arrays (afv_forest_set_var / get_var) by kernel
 * loads and stores over the host link, without the device staging buffer;
 * 0 copies through the staging buffer with the copy engines, which leaves
 * the SMs to other work (another forest's solve) during the transfer.
 * AFV_OPT_DEFECT_CELLS: cells per thread of the fixed-point defect (1, 2 or
 * 4: a block of 256 threads takes 256 / (cells / this) leaves of a small box
 * shape at a time, at least 16 threads per leaf, within 48 KB of shared
 * memory), 0 (default) the most of 4, 2, 1 that the box shape allows; the
 * same values for every setting. afv_forest_autotune_all sets it. */
enum {
  AFV_OPT_SWEEP_KERNEL = 0,
  AFV_OPT_GRAPHS = 1,
  AFV_OPT_RESTRICT_KERNEL = 2,
  AFV_OPT_SMALL_SWEEPS = 3,
  AFV_OPT_PROFILE_LEAD_US = 4,
  AFV_OPT_DEFECT_KERNEL = 5,
  AFV_OPT_COARSE_END = 6,
  AFV_OPT_WAIT_LIMIT_US = 7,
  AFV_OPT_DIRECT_BOXES = 8,
  AFV_OPT_ZERO_COPY = 9,
  AFV_OPT_DEFECT_CELLS = 10
};
int afv_forest_set_option(afv_forest* f, int option, int value);
int afv_forest_get_option(afv_forest* f, int option, int* value);
/* No counterpart in the reference: times the sweep kernel variants on this
 * forest (two FP32 correction V-cycles each on the mixed-precision scratch
 * state; needs mixed_buffers) and sets AFV_OPT_SWEEP_KERNEL to the fastest.
 * choice receives it; ms3 (may be NULL) the ms per V-cycle of variants 1, 2
 * and 0 in that order. */
int afv_forest_autotune(afv_forest* f, int* choice, float* ms3);
/* No counterpart in the reference: the full tuning pass. Times the six sweep
 * kernels (AFV_OPT_SWEEP_KERNEL 0..5: the block-pipelined level kernel, the
 * warp-per-box kernel with bulk copies in four warp / stage shapes, the one
 * with per-lane copies), keeps the fastest, then times AFV_OPT_SMALL_SWEEPS
 * and AFV_OPT_COARSE_END on and off with it and keeps the fastest pair.
 * choice3 receives (sweep kernel, small sweeps, coarse end); ms10 (may be
 * NULL) the ms per FP32 V-cycle of sweep kernels 0..5, then of the (small,
 * coarse end) settings (0,0), (0,1), (1,0), (1,1). Last it times the
 * fixed-point defect's cells per thread as afv_forest_autotune_defect does
 * and keeps the fastest (AFV_OPT_DEFECT_CELLS). Needs mixed_buffers. */
int afv_forest_autotune_all(afv_forest* f, int* choice3, float* ms10);
/* No counterpart in the reference: times the mixed solve's fixed-point defect
 * with 1, 2 and 4 cells per thread (five launches each on the current state;
 * it writes only the correction's right-hand side and the norms, which every
 * solve recomputes) and sets AFV_OPT_DEFECT_CELLS to the fastest. cells
 * receives it; ms3 (may be NULL) the ms per launch of 1, 2 and 4, -1 for a
 * shape the forest's boxes do not allow (and all three -1 with
 * AFV_OPT_DEFECT_KERNEL 0). Needs mixed_buffers. */
int afv_forest_autotune_defect(afv_forest* f, int* cells, float* ms3);

/* No counterpart in the reference: the profiled event pairs one by one (up
 * to max; n_total receives how many were recorded): kernel kind, level,
 * device time in ms, algorithmic bytes and the launches the pair covers
 * (the consecutive half-sweeps of a level share one pair). */
int afv_forest_profile_entries(afv_forest* f, long long max, int* kind, int* level, double* ms,
                               double* algorithmic_bytes, int* launches, long long* n_total);

#ifdef __cplusplus
}
#endif
#endif /* AFIVO_GB300_H */
