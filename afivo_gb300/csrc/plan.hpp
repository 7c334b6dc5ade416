// Device layout of a forest of trees, built on the host.
//
// Slots number all boxes of all trees: level by level from the coarsest, then
// tree by tree, then in Morton order of the box index (the order a$D_tidy_up
// gives ids, src/m_aX_core.f90:267-292). With that order the 2^D children of a
// parent at level >= 1 sit in consecutive slots in child-number order, so a
// slot stores only its first child. Cell data of slot s lives at offg[s]
// ((nc+2)^D values, phi and tmp) and offi[s] (nc^D values, rhs).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "desc.hpp"
#include "host_tree.hpp"

namespace afv {

struct BcSpec {
  int type = AFV_BC_DIRICHLET;  // AFV_BC_DIRICHLET / AFV_BC_NEUMANN
  int src_lpl = 0;
  std::vector<double> gauss;    // empty: boundary value 0
  // Per-face records given by the caller instead (a sampled sides_bc hook):
  // one type per physical face and nc^(D-1) values per face, faces in the
  // host exchange order (boxes of the level lists, faces low x first).
  bool per_face = false;
  std::vector<int> face_type;
  std::vector<double> face_vals;
};

struct Plan {
  int dim = 2, nc = 8, min_lvl = 1, max_lvl = 1, n_trees = 0, n_slots = 0;
  int cyl = 0;  // the trees' coordinates are cylindrical (2-D)
  // per slot
  std::vector<int> nb;           // [s*2D+f]: slot, -1 refinement boundary, -2 physical
  std::vector<int> parent;       // slot or -1
  std::vector<int> first_child;  // slot or -1
  std::vector<int> tree;         // tree index
  std::vector<int> lvl;          // level
  std::vector<int> qd;           // child-number bits within the parent (lvl >= 2), else -1
  std::vector<int> host_id;      // id in its host tree
  std::vector<int> ix;           // [s*D+d]
  std::vector<double> dr;
  std::vector<double> r_min;     // [s*D+d]
  std::vector<long long> offg, offi;
  std::vector<long long> nbo;    // [s*2D+f] offg of the neighbour / of the parent at a refinement boundary
  std::vector<int> bctype;       // [s*2D+f]
  std::vector<long long> bcoff;  // [s*2D+f]
  std::vector<double> bcval;
  long long n_elem_g = 0, n_elem_i = 0;
  // per level (index lvl - min_lvl): slot range and leaf / parent lists
  std::vector<int> lvl_lo, lvl_n;
  std::vector<std::vector<int>> leaves, parents;
  std::vector<int> all_leaves;  // leaves of every level (all have n_cell = nc), tree by tree
  // Counts over the trees before t, for solves of the first t trees only:
  // [L * (n_trees + 1) + t] slots, leaves and parents of level index L
  // (within a level the slots, and so the lists, are tree-major), and
  // [t] entries of all_leaves.
  std::vector<int> lvl_tprefix, leaves_tprefix, parents_tprefix, all_leaves_tprefix;
  // per tree: slots in the tree's level-list order (the host exchange order)
  std::vector<std::vector<int>> host_order;
  std::vector<int> tree_highest;
  std::vector<long long> tree_leaf_cells;
  std::vector<BcSpec> bc;
  std::vector<SlotDesc> desc;   // per slot, see desc.hpp
  std::vector<long long> nbo2;  // [s*2D+f] refinement boundary: offg of the parent's neighbour

  int nc_at(int l) const { return l >= 1 ? nc : (nc >> (1 - l)); }
  int L(int l) const { return l - min_lvl; }
};

// Build the plan; returns AFV_OK or AFV_ERR_INVALID with a message.
int build_plan(const std::vector<const HostTree*>& trees, Plan& p, std::string& err);

// (Re)compute the boundary value records of one tree from its BcSpec.
void plan_fill_bc(Plan& p, int tree);

// (Re)build the per-slot descriptors (after the tables or the boundary values change).
void plan_build_desc(Plan& p);

// Number of physical-boundary faces of one tree and of their face cells.
void plan_count_bc_faces(const Plan& p, int tree, long long& n_faces, long long& n_values);

}  // namespace afv
