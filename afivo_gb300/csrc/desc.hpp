// Per-slot descriptor: everything a kernel needs to know about one box, in
// one 128-byte record that a bulk copy brings into shared memory together
// with the box's cells.
#pragma once
#include <cstddef>

namespace afv {

// Face codes of a slot descriptor.
enum : signed char {
  kFaceRefinement = -1,  // no box on this level: coarse neighbour (refinement boundary)
  kFaceDirichlet = -2,   // physical boundary, Dirichlet
  kFaceNeumann = -3,     // physical boundary, Neumann
};

struct alignas(16) SlotDesc {
  long long nbo[6];    // per face: offg of the neighbour (code >= 0) or of the parent
                       // (refinement boundary), or the offset of the boundary values
                       // (physical boundary; -1 = zero values)
  signed char code[6]; // per face: 0 neighbour box, or one of the kFace* codes
  short pad0;
  int qd;              // child-number bits within the parent (levels >= 2), else -1
  int tree;
  double dr;           // cell size
  double dx2;          // dr * dr
  double inv_dx2;      // 1 / (dr * dr)
  long long offg;      // this box's ghosted storage
  long long offi;      // this box's interior storage
  float drf;           // (float) dr
  float dx2f;          // (float) (dr * dr)
  float inv_dx2f;      // 1.0f / (float) (dr * dr)
  int first_child;
  int parent;
  int pad1;
};
static_assert(sizeof(SlotDesc) == 128, "SlotDesc must be 128 bytes");
// Kernels read these fields as 32-bit words (word = byte offset / 4).
static_assert(offsetof(SlotDesc, nbo) == 0 && offsetof(SlotDesc, code) == 48 &&
                  offsetof(SlotDesc, qd) == 56 && offsetof(SlotDesc, tree) == 60,
              "SlotDesc field offsets");

}  // namespace afv
