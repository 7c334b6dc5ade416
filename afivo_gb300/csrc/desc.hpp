// Per-slot descriptor: everything a kernel needs to know about one box, in
// one 128-byte record that a bulk copy brings into shared memory together
// with the box's cells.
#pragma once

namespace afv {

struct alignas(16) SlotDesc {
  long long nbo[6];  // per face: offg of the neighbour (code >= 0) or of the parent (code -1),
                     // or the offset of the boundary values (codes -2/-3, -1 = zero values)
  int code[6];       // per face: >= 0 neighbour slot, -1 refinement boundary,
                     // -2 Dirichlet boundary, -3 Neumann boundary
  int qd;            // child-number bits within the parent (levels >= 2), else -1
  int tree;
  double dr;
  long long offg;    // this box's ghosted storage
  long long offi;    // this box's interior storage
  int first_child;
  int parent;
  int pad[4];
};
static_assert(sizeof(SlotDesc) == 128, "SlotDesc must be 128 bytes");

}  // namespace afv
