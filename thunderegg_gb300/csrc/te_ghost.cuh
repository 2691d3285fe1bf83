// te_ghost.cuh -- ghost-filling tables and device helpers shared by the
// ghost-fill kernel and the fused operator kernels.
#pragma once
#include "te_internal.cuh"

namespace te {

// Geometry of one face (Face<D,M>) of a padded patch, in cells of one
// component: where its interior slice and ghost slice start, how to step
// inward (one step per side the face lies on) and along its tangential axes.
// (PatchView::getSliceOn / getGhostSliceOn, PatchView.h:100-240)
struct FaceGeom {
  int ibase;      // interior slice, depth 0, tangential coords 0
  int gbase;      // ghost slice, layer 0, tangential coords 0
  int inward[3];  // per side of the face: +stride (lower side) / -stride (upper side)
  int tstride[2]; // tangential strides
  int nt[2];      // tangential sizes (1 if absent)
  int nsides;     // D - M
};

struct FaceTable {
  FaceGeom f[26];  // by slot (Face<D,M>::sum_of_faces + index)
};

// One ghost region to write: face (M, face) of `patch`.
struct GSlab {
  int patch;
  int call0;     // first incoming call in the call table
  int8_t M, face;
  int8_t own_type;  // this patch's neighbour type on the face (-1 none)
  int8_t own_orth;  // orth_on_coarse when own_type is Coarse
  int8_t zero;      // ghosts zeroed first (the patch has a neighbour on the face)
  int8_t ncalls;    // incoming fillGhostCellsFor*NbrPatch calls, in reference order
  int8_t pad[2];
};
// A neighbour's call that writes into this slab: the caller patch, its face
// (the opposite of the slab's face), the neighbour type as the caller sees
// it and the orthant it passes.
struct GCall {
  int src;
  int8_t type, orth, src_face, pad;
};
// Everything the gather of one side of one patch needs, in one record
// (te_ghost_filler::d_side_rec, [P * 2D]): the side's code as in d_side_code and,
// for a side with a slab, the slab's own term and its incoming calls inline, so
// a gather costs one record load before the neighbours' values instead of a
// chain code -> slab -> call -> values.  A slab with more than kSideRecCalls
// calls (none arise from a 2:1 balanced mesh) keeps ncalls = -1: its gather
// reads the slab table.
constexpr int kSideRecCalls = 4;
struct __align__(16) SideRec {
  int code;
  int8_t own_type, own_orth, zero, ncalls;
  GCall calls[kSideRecCalls];
  int pad[2];
};

FaceTable make_face_table(const Layout& L);
int slot_of(int D, int M, int face);
int face_opposite(int D, int M, int v);

}  // namespace te

struct te_ghost_filler {
  const te_domain* dom = nullptr;
  int scheme = 0, fill_type = 0;
  std::vector<std::array<int, 6>> calls;  // reference call list
  std::vector<te::GSlab> h_slabs;
  std::vector<int> h_slab_start;          // [P+1]
  te::DevBuf<te::GSlab> d_slabs;
  te::DevBuf<te::GCall> d_calls;
  te::DevBuf<int> d_slab_start;
  // [P * 2D] per patch side: >= 0 the ghosts are a plain copy of that patch's
  // face (a Normal neighbour and no own term), -1 no neighbour, <= -2 the
  // side's slab is -2 - code
  te::DevBuf<int> d_side_code;
  te::DevBuf<te::SideRec> d_side_rec;  // [P * 2D] the same sides with their slabs inline
  bool other_slabs = false;  // slabs beyond d_side_code (edges, corners, sides without a neighbour)
  te::FaceTable faces;
};

namespace te {
// fill ghosts of a level buffer (all patches)
void ghost_fill(const te_ghost_filler* g, int nc, int dtype, void* u, cudaStream_t s);
}
