// teref_domain.hpp -- TEST INFRASTRUCTURE ONLY: ThunderEgg Domain<D> objects and
// unmanaged Vector<D> views built from the flat level tables of include/te_gpu.h,
// shared by the reference driver (teref.cpp) and the adapter driver
// (adapters_drive.cpp).  Include after the ThunderEgg headers.
#pragma once

#include <ThunderEgg/Domain.h>
#include <ThunderEgg/Vector.h>

#include <array>
#include <vector>

#include "te_gpu.h"

namespace teref_tables {
using namespace ThunderEgg;

inline int slots(int D) { return D == 2 ? 8 : 26; }

template <int D, int M>
inline void set_face_nbrs(PatchInfo<D>& pi, const te_level_desc* d, int p, int slot0) {
  for (int f = 0; f < (int)Face<D, M>::number_of; f++) {
    int slot = slot0 + f;
    size_t k = (size_t)p * slots(D) + slot;
    int t = d->nbr_type[k];
    const int* ids = d->nbr_ids + k * 4;
    Face<D, M> face((unsigned char)f);
    if (t == TE_NBR_NORMAL) {
      pi.setNbrInfo(face, new NormalNbrInfo<M>(ids[0]));
    } else if (t == TE_NBR_COARSE) {
      pi.setNbrInfo(face, new CoarseNbrInfo<M>(ids[0], Orthant<M>((unsigned char)d->nbr_orth[k])));
    } else if (t == TE_NBR_FINE) {
      std::array<int, Orthant<M>::num_orthants> a;
      for (size_t i = 0; i < a.size(); i++) a[i] = ids[i];
      pi.setNbrInfo(face, new FineNbrInfo<M>(a));
    }
  }
}

template <int D>
inline Domain<D> make_domain(const te_level_desc* d, int domain_id = 0) {
  std::vector<PatchInfo<D>> pinfos(d->num_patches);
  std::array<int, D> ns;
  for (int a = 0; a < D; a++) ns[a] = d->ns[a];
  for (int p = 0; p < d->num_patches; p++) {
    PatchInfo<D>& pi = pinfos[p];
    pi.id = d->id[p];
    pi.rank = 0;
    pi.refine_level = d->refine_level[p];
    pi.parent_id = d->parent_id[p];
    pi.parent_rank = d->parent_id[p] >= 0 ? 0 : -1;
    pi.orth_on_parent = d->orth_on_parent[p] >= 0 ? Orthant<D>((unsigned char)d->orth_on_parent[p])
                                                  : Orthant<D>::null();
    for (int c = 0; c < (1 << D); c++) {
      pi.child_ids[c] = d->child_ids[(size_t)p * (1 << D) + c];
      pi.child_ranks[c] = pi.child_ids[c] >= 0 ? 0 : -1;
    }
    pi.num_ghost_cells = d->num_ghost;
    pi.ns = ns;
    for (int a = 0; a < D; a++) {
      pi.starts[a] = d->starts[(size_t)p * D + a];
      pi.spacings[a] = d->spacings[(size_t)p * D + a];
    }
    if constexpr (D == 2) {
      set_face_nbrs<2, 0>(pi, d, p, 0);
      set_face_nbrs<2, 1>(pi, d, p, 4);
    } else {
      set_face_nbrs<3, 0>(pi, d, p, 0);
      set_face_nbrs<3, 1>(pi, d, p, 8);
      set_face_nbrs<3, 2>(pi, d, p, 20);
    }
  }
  return Domain<D>(Communicator(MPI_COMM_WORLD), domain_id, ns, d->num_ghost, pinfos.begin(),
                   pinfos.end());
}

// Vector aliasing a caller buffer (Vector.h:199-215, unmanaged constructor)
template <int D>
inline Vector<D> wrap(const Domain<D>& dom, int nc, double* data) {
  std::array<int, D + 1> strides, lengths;
  int st = 1;
  for (int a = 0; a < D; a++) {
    strides[a] = st;
    lengths[a] = dom.getNs()[a];
    st *= dom.getNs()[a] + 2 * dom.getNumGhostCells();
  }
  strides[D] = st;
  lengths[D] = nc;
  long ps = (long)st * nc;
  std::vector<double*> starts(dom.getNumLocalPatches());
  for (size_t i = 0; i < starts.size(); i++) starts[i] = data + i * ps;
  return Vector<D>(Communicator(MPI_COMM_WORLD), starts, strides, lengths, dom.getNumGhostCells());
}

}  // namespace teref_tables
