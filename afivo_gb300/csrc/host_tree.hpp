// Host-side quadtree/octree of NxN(xN) blocks: the index work that feeds the
// device solver. Restates the reference's tree build bit for bit
// (src/m_aX_core.f90:24-787, src/m_morton.f90), in a structure-of-arrays form
// that the device planner (forest.cpp) reads directly.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "afivo_gb300.h"

namespace afv {

// Refinement flags and sentinels, src/m_aX_t.f90:17-49
enum : int {
  kRmRef = -1,
  kKeepRef = 0,
  kDoRef = 1,
  kDerefine = -2,
  kRefine = 2,
  kNoBox = 0,
};

struct LevelLists {
  std::vector<int> ids, leaves, parents;
};

// Geometry helpers shared by the tree builder and the planner.
inline int child_bit(int c0, int d) { return (c0 >> d) & 1; }  // c0 = child number - 1

// Morton key of a 0-based index, src/m_morton.f90:33-59
uint64_t morton_key(int dim, const int* ix0);

class HostTree {
 public:
  int dim = 2;
  int coord = 0;  // 0 Cartesian, 1 cylindrical (a$D_init's coord, src/m_aX_core.f90:58-70)
  int nch = 4;  // 2^dim
  int nnb = 4;  // 2*dim
  int n_cell = 8;
  int min_lvl = 1;
  int lvl_limit = 30;
  int box_limit = 0;
  int highest_lvl = 0;
  int highest_id = 0;
  bool ready = false;
  int n_adjust = 0;  // adjust_refinement passes done (keys the seeded criteria)
  double dr_base = 0;
  double r_base[3] = {0, 0, 0};

  // Per box id (index 0 unused): structure of arrays.
  std::vector<int> lvl, parent, ncell, in_use;
  std::vector<int> ix;         // [id*dim + d]
  std::vector<int> children;   // [id*nch + c]
  std::vector<int> neighbors;  // [id*nnb + nb]
  std::vector<double> dr;
  std::vector<double> r_min;   // [id*dim + d]

  std::vector<LevelLists> levels;  // index lvl - min_lvl, lvl = min_lvl..lvl_limit+1

  LevelLists& L(int l) { return levels[l - min_lvl]; }
  const LevelLists& L(int l) const { return levels[l - min_lvl]; }
  int capacity() const { return (int)lvl.size() - 1; }
  int n_used() const;
  bool has_children(int id) const { return children[(size_t)id * nch] != kNoBox; }
  int ichild_of(int id) const;
  int n_cell_at(int l) const { return l >= 1 ? n_cell : (n_cell >> (1 - l)); }

  int init(int dim, int n_cell, double dr, const double* r_min, int lvl_limit, int coarsen_to,
           double mem_limit_gb, std::string& err);
  int set_base(int n_boxes, const int* ix_list, int* nb_list, std::string& err);
  // One pass of a$D_adjust_refinement. fn is called for every leaf and for
  // the parent of every first child, like the reference's ref_subr.
  int adjust(afv_ref_fn fn, void* user, int* n_add, int* n_rm, std::string& err);

 private:
  void resize(int new_size);
  void get_free_ids(int n, int* out);
  void lists_of(LevelLists& lv);
  void tidy_up(double max_hole_frac, int n_clean_min);
  int consistent_flags(std::vector<int>& flags, afv_ref_fn fn, void* user, std::string& err);
  void add_children(int id, const int* c_ids);
  void remove_children(int id);
  void set_neighbs(int id);
  int find_neighb(int id, int nb) const;
  void make_view(int id, afv_box_view* v) const;
};

// Built-in refinement criteria (a C callback + its parameters).
struct BuiltinCrit {
  afv_ref_crit c;
  std::vector<double> gauss;
  int dim;
  const HostTree* tree;
};
void builtin_ref_fn(const afv_box_view* box, int* ref_flag, void* user);

// Source functions used for right-hand sides, criteria and boundary values.
double source_eval(int dim, int lpl, const double* gauss, int n_gauss, const double* r);

}  // namespace afv
