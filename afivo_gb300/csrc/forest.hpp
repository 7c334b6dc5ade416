// Device-resident forest: the plan's tables and the cell data on one GPU, and
// the multigrid drivers that sweep it (one launch per level and operator for
// all trees at once).
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "plan.hpp"

namespace afv {

namespace opdev {
struct Op;
}
namespace dev {
struct BoxSet;
}
using dev_BoxSet = dev::BoxSet;

template <class T>
struct Arrays {
  T* phi = nullptr;  // ghosted
  T* rhs = nullptr;  // interior
  T* tmp = nullptr;  // ghosted
};

struct DevMeta {
  int* parent = nullptr;
  int* first_child = nullptr;
  int* tree = nullptr;
  long long* offg = nullptr;
  long long* offi = nullptr;
  double* bcval = nullptr;
  int* active = nullptr;  // [n_trees]
  SlotDesc* desc = nullptr;
  long long* nbo2 = nullptr;
  int* err = nullptr;  // device error word (bounded waits)
  double* rmin = nullptr;  // [slot*D + d] lower corner of the box
  // clock cycles a kernel's wait for one of its copies may take before it
  // gives up (AFV_OPT_WAIT_LIMIT_US; about two seconds by default)
  long long wait_limit = 4000000000LL;
};

struct MgOpts {
  int n_down = 2, n_up = 2, n_base = 2;
};

// Kernel kinds for the event profiler (afv_forest_profile).
enum ProfKind {
  kProfSweep = 0,
  kProfFill,
  kProfRestrict,
  kProfCoarseRhs,
  kProfCorrect,
  kProfResidual,
  kProfDefect,
  kProfAccumulate,
  kProfCoarseEnd,
  kProfOther,
  kProfKinds
};

struct ProfEntry {
  cudaEvent_t start, stop;
  int kind;
  int level;     // level the launch works on (parents' level for coarse_rhs / correct)
  double bytes;  // algorithmic bytes of the launches
  int count;     // launches between the two events (consecutive half-sweeps share a pair)
};

struct SolveStats {
  std::vector<int> cycles;
  std::vector<double> rel_res;
  int status = 0;
};

class Forest {
 public:
  Plan plan;
  int device = 0;
  int n_sm = 148;
  int sweep_kernel = 1;  // 0: block-pipelined k_level_tma, 1: warp-per-box k_sweep_warp, 2: its async variant
  bool use_restrict_warp = true;  // warp-per-box restriction on levels >= 2
  bool defect_fx = true;          // mixed defect: fixed-point Laplacian (false: FP64 sum)
  int defect_cells = 0;           // its cells per thread (1, 2, 4; 0: the default per box shape)
  bool use_coarse_end = true;     // correction cycle's levels l0..1 in one launch (k_coarse_end)
  int coarse_end_levels = -1;     // levels k_coarse_end covers (0: not eligible; -1: not yet known)
  int coarse_end_depth(int highest);
  void coarse_end(const Arrays<float>& a, const MgOpts& mg, int nl);
  // All half-sweeps of a level in one block (k_sweep_small) when the level has
  // at most kSmallCells interior cells: measured faster than one launch per
  // half-sweep for 512 cells (8.5 us for four half-sweeps against 14 us),
  // slower for 4096 (19.8 us against 16.3 us).
  bool use_small_sweeps = true;
  // Levels of at most this many boxes take the unstaged half-sweep
  // (k_sweep_direct); -1: FP64 sweeps on every level (FP64 solves 1.3 to
  // 3 % faster on the 3-D and batched 2-D workloads), FP32 sweeps never (the
  // staged warp sweep is as fast there).
  int direct_boxes = -1;
  bool zero_copy = true;  // host exchange of pinned memory by SM loads and stores, no staging buffer
  template <class T> int direct_limit() const {
    return direct_boxes >= 0 ? direct_boxes : (sizeof(T) == 8 ? (1 << 30) : 0);
  }
  static constexpr long long kSmallCells = 2048;
  static constexpr long long kSmallSmemBytes = 200 * 1024;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // second branch of an iteration (fork / join)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void fork();
  void join();
  DevMeta meta;
  Arrays<double> d64;
  Arrays<float> d32;
  double* base_phi64 = nullptr;  // FP64 copy of the coarsest level for the mixed cycle
  double* base_rhs64 = nullptr;
  bool mixed = false;
  // level lists on the device
  // Variables beyond phi, rhs and tmp (afv_forest_add_vars): ghosted FP64
  // cell-centred variables numbered 3, 4, ... in phi's layout, and face
  // variables, per slot D blocks of (nc+1) * nc^(D-1) values (fx, fy, fz),
  // at fc + (ifc * n_slots + slot) * fc_stride.
  std::vector<double*> xcc;
  int n_fc = 0;
  double* fc = nullptr;
  long long fc_stride = 0;
  // Slot tables the general utilities read, uploaded on first use: the
  // neighbour slot per face (-1 refinement boundary, -2 physical), level and
  // child-number bits per slot.
  int* d_nb = nullptr;
  int* d_lvl = nullptr;
  int* d_qd = nullptr;
  // Operator of the FP64 multigrid routines (afv_mg_set_operator): AFV_OP_LPL
  // (the fused constant-coefficient kernels in Cartesian trees), or one of
  // AFV_OP_LPLD, AFV_OP_CLPL, AFV_OP_CLPLD, AFV_OP_LPLLSF, AFV_OP_AUTO (the
  // generic kernels of operators.cu, with eps in cell variable i_eps, the
  // level set and its boundary value in i_lsf / i_bval, and the per-box tags
  // of the auto dispatch in d_tags).
  int op = AFV_OP_LPL;
  int i_eps = -1, i_lsf = -1, i_bval = -1;
  int* d_tags = nullptr;
  int* d_ix = nullptr;  // [slot*D + d] the boxes' ix (cylindrical radial factors)
  // eps_0 eps_f / (eps_0 + eps_f) per interior cell and face (the lpld
  // operators' face weights, [(offi + q) * 2D + f]), taken with the operator
  double* d_coef = nullptr;
  int set_operator(int new_op, int new_i_eps, int new_i_lsf, int new_i_bval, std::string& err);
  const double* eps_ptr() const;
  void gen_coef();
  opdev::Op op_args() const;  // what the generic kernels read
  // The FP64 routines take the generic kernels of operators.cu: an operator
  // other than the Laplacian, or cylindrical coordinates (whose restriction
  // is weighted).
  bool generic() const { return op != AFV_OP_LPL || plan.cyl; }
  void gen_init_phi_rhs();  // init_phi_rhs (FMG without a guess)
  void gen_gsrb_boxes(int lvl, int n_cycle);
  void gen_update_coarse(int lvl, bool copy_tmp);
  void gen_correct(int lvl_parent);
  void gen_residual(int lvl, unsigned long long* norm);
  void gen_vcycle(const MgOpts& mg, int highest, bool set_residual);
  void fill64(int lvl);  // ghost fill of the FP64 phi of a level (mg sides_rb, sides_bc)
  int n_cc_vars() const { return 3 + (int)xcc.size(); }
  // Device array of cell variable iv (0 phi, 1 rhs, 2 tmp, 3.. extra).
  double* var_ptr(int iv) const {
    if (iv == 0) return d64.phi;
    if (iv == 1) return d64.rhs;
    if (iv == 2) return d64.tmp;
    return (iv >= 3 && iv < n_cc_vars()) ? xcc[iv - 3] : nullptr;
  }
  int* d_lists = nullptr;
  std::vector<int> leaves_off, parents_off;  // offsets in d_lists per level
  int all_leaves_off = 0;
  // per-tree reductions
  unsigned long long* d_norm = nullptr;  // [n_trees * kStripes] striped per-tree maxima
  unsigned long long* d_red = nullptr;   // [n_trees] reduced maxima
  double* d_fmax = nullptr;              // [n_trees]
  // [4]: active trees after the last check, the error word at that check,
  // iterations of the current solve (graph loop), unused
  int* d_count = nullptr;
  int* d_failed = nullptr;               // [n_trees] nonzero: residual not finite
  int* d_solve_mask = nullptr;           // [n_trees] trees a solve takes part in
  int* h_solve_mask = nullptr;           // pinned [n_trees]
  int* d_cycles = nullptr;               // [n_trees] V-cycles of the current solve
  unsigned long long* d_final = nullptr; // [n_trees] residual norm at the tree's last check (double bits)
  int* h_count = nullptr;                // pinned [4]: copy of d_count
  unsigned long long* h_norm = nullptr;  // pinned [n_trees]
  // pinned results of a solve, copied once at its end
  int* h_cycles = nullptr;               // [n_trees]
  unsigned long long* h_final = nullptr; // [n_trees]
  int* h_failed = nullptr;               // [n_trees]
  double* h_fmax = nullptr;              // [n_trees]
  bool readback = true;  // each residual check copies d_count to h_count (host-driven solve loop)
  double* d_stage = nullptr;             // staging for host exchange
  long long stage_elems = 0;
  int* d_stage_slots = nullptr;          // every tree's host-order slots, concatenated
  // host exchange plan, made on the first exchange: per tree the interior
  // and ghosted value counts, the runs of boxes of one level, and where its
  // slots start in d_stage_slots
  struct XferRun {
    int first, n, lvl;
  };
  bool xfer_ready = false;
  std::vector<std::array<long long, 2>> xfer_total;
  std::vector<std::vector<XferRun>> xfer_runs;
  std::vector<long long> xfer_order_off;
  long long bytes = 0;
  std::vector<int> host_active;
  // CUDA graph of a whole solve, per precision, keyed by the options: set-up,
  // a conditional while node over the iterations (body captured on
  // loop_stream), finish; the kernels each part launches
  struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    long long k_pre = 0, k_body = 0, k_post = 0;
    int n_down = -1, n_up = -1, n_base = -1, max_cycles = -1;
    double tol = -1;
  };
  std::map<long long, GraphCache> graphs;  // by precision and tree_limit
  GraphCache& graph_for(int precision, int limit) {
    const long long key = (long long)limit * 2 + (precision == AFV_PREC_MIXED ? 1 : 0);
    if (graphs.size() >= 32 && !graphs.count(key)) drop_graphs();  // bound the cache (many prefix lengths)
    return graphs[key];
  }
  cudaStream_t loop_stream = nullptr;
  bool use_graphs = true;
  void drop_graphs();
  // event profiler: when enabled, launches of the selected kinds (bit mask)
  // are bracketed by CUDA events on the forest's stream
  int prof_mask = 0;
  int prof_level = 0;  // level tag of the next profiled launches
  int prof_lead_us = 0;  // > 0: each profiled solve iteration starts behind a k_hold of this length
  // Consecutive half-sweeps of one level are timed by one pair of events
  // (a group), so the events' own cost is not charged to every launch.
  bool group_on = false;
  double group_bytes = 0;
  int group_count = 0;
  long long n_launches = 0;  // every kernel launched on the stream
  std::vector<ProfEntry> prof;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t prof_begin(int kind);
  void prof_end(cudaEvent_t start, int kind, double bytes, int count = 1);
  int prof_read(int kind, long long* launches, double* ms, double* bytes);
  long long prof_entries(long long max, int* kind, int* level, double* ms, double* bytes, int* count);
  void prof_reset();

  ~Forest();
  int create(const std::vector<const HostTree*>& trees, const afv_forest_opts* opts, std::string& err);
  int upload_bc(std::string& err);

  // Host exchange in the reference's box layout.
  int set_var(int tree, int var, const double* host, int interior_only, std::string& err);
  int get_var(int tree, int var, double* host, int interior_only, std::string& err);

  // Activity masks.
  int set_active_all(int v);
  int set_active_host(const std::vector<int>& a);

  // Multigrid (FP64 state).
  int gsrb_level(int lvl, int n_cycle, std::string& err);
  int fill_level(int lvl, std::string& err);
  int update_coarse(int lvl, std::string& err);
  int correct_children(int lvl_parent, std::string& err);
  int residual_all(unsigned long long* norm, std::string& err);
  int vcycle(const MgOpts& mg, int highest, bool set_residual, std::string& err);
  int autotune(int* choice, float* ms3, std::string& err);
  int autotune_all(int* sweep, int* small, int* coarse_end, float* ms10, std::string& err);
  int set_source_device(int tree, int lpl, int n_gauss, const double* gauss, std::string& err);
  int fmg(const MgOpts& mg, bool set_residual, bool have_guess, std::string& err);
  int gc_tree(std::string& err);
  int max_abs(int tree, int var, double* out, std::string& err);
  // max_abs with its scratch in static device memory (noalloc.cuh)
  int max_abs_static(int tree, int var, double* out, std::string& err);
  // mask (n_trees entries, may be null = every tree): the trees the solve
  // takes part in; the others are left as they are
  int solve(const MgOpts& mg, int precision, double tol, int max_cycles, SolveStats& st,
            std::string& err, const int* mask = nullptr);
  int zero_tree(int tree, int var, std::string& err);

  // Generic-precision pieces.
  template <class T> void sweep(const Arrays<T>& a, int lvl, int n, bool pull, bool homog);
  template <class T> void fill(const Arrays<T>& a, int lvl, bool homog);
  template <class T> void restrict_res(const Arrays<T>& a, int lvl, bool with_res, bool pull = false,
                                       bool homog = false);
  template <class T> void coarse_rhs(const Arrays<T>& a, int lvl_parent, bool copy_tmp,
                                     bool pull = false, bool homog = false);
  template <class T> void correct(const Arrays<T>& a, int lvl_parent, bool pull = false, bool homog = false);
  template <class T> void residual(const Arrays<T>& a, int lvl, unsigned long long* norm, bool store);
  template <class T> void gsrb_boxes(const Arrays<T>& a, int lvl, int n_cycle, bool homog);
  template <class T> void update_coarse_t(const Arrays<T>& a, int lvl, bool homog, bool copy_tmp);
  template <class T> bool sweeps_small(const Arrays<T>& a, int lvl, int n_first, int n_count, bool pull_first,
                                       bool homog);
  template <class T> void vcycle_t(const Arrays<T>& a, const MgOpts& mg, int highest, bool homog,
                                   bool base64, bool inner = false);
  template <class T> void fill_set(const Arrays<T>& a, int lvl, dev_BoxSet bs, bool homog);
  void fill_all64(bool homog);
  // Enqueue (no host synchronisation) one solve iteration / its residual
  // check (count_cycle: the check follows a cycle), the solve's set-up (with
  // a loop handle: the loop-entry decision) and its finish.
  void enqueue_iteration(const MgOpts& mg, int precision, double tol);
  void enqueue_residual_check(int precision, double tol, int count_cycle = 1);
  void launch_defect();
  int defect_shapes() const;
  int defect_cr() const;
  void tune_defect(cudaEvent_t e0, cudaEvent_t e1, float* ms3);
  int autotune_defect(int* cells, float* ms3, std::string& err);
  void enqueue_solve_begin(int precision, double tol, int max_cycles, const cudaGraphConditionalHandle* h);
  void enqueue_solve_end(int precision);
  int build_solve_graph(GraphCache& gc, const MgOpts& mg, int precision, double tol, int max_cycles,
                        std::string& err);
  void restrict_tree_phi64();

  int check(std::string& err, const char* where);
  int check_device_error(std::string& err);  // reads and clears the device error word
  void norm_reset();
  void norm_fold();  // d_norm -> d_red
  // Solves of the first tree_limit trees only (0: all): the level sets and
  // lists below then hold those trees' boxes, a prefix of each (a solve whose
  // mask selects leading trees sets it, see solve()).
  int tree_limit = 0;
  int lvl_n(int l) const {
    if (l < plan.min_lvl || l > plan.max_lvl) return 0;
    return tree_limit ? plan.lvl_tprefix[(size_t)plan.L(l) * (plan.n_trees + 1) + tree_limit] : plan.lvl_n[plan.L(l)];
  }
  int n_all_leaves() const {
    return tree_limit ? plan.all_leaves_tprefix[tree_limit] : (int)plan.all_leaves.size();
  }
  int n_trees_run() const { return tree_limit ? tree_limit : plan.n_trees; }
  void zero_correction(cudaStream_t st);  // the FP32 phi of the trees in the run
  int* leaves_list(int l) { return d_lists + leaves_off[plan.L(l)]; }
  dev_BoxSet level_set(int l) const;  // all boxes of level l (a slot range)
  int* parents_list(int l) { return d_lists + parents_off[plan.L(l)]; }
  int n_leaves(int l) const {
    return tree_limit ? plan.leaves_tprefix[(size_t)plan.L(l) * (plan.n_trees + 1) + tree_limit]
                      : (int)plan.leaves[plan.L(l)].size();
  }
  int n_parents(int l) const {
    if (l < plan.min_lvl || l > plan.max_lvl) return 0;
    return tree_limit ? plan.parents_tprefix[(size_t)plan.L(l) * (plan.n_trees + 1) + tree_limit]
                      : (int)plan.parents[plan.L(l)].size();
  }
  // First and last slot of tree t on level l ({-1, -1}: none); a level's
  // slots are tree-major, so a tree's are contiguous. The table is built on
  // first use.
  std::pair<int, int> tree_level_range(int t, int l);
  std::vector<int> tl_first, tl_last;  // [t * levels + (l - min_lvl)]
};

}  // namespace afv
