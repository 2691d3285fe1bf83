// te_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A plain CPU restatement of ThunderEgg's geometric-multigrid hot path, used
// as the checker for the CUDA path (tests/, __graft_entry__.smoke()) and as
// the timed CPU baseline of bench.py.  Nothing in the product links, loads or
// calls this file.  Each function cites the ThunderEgg source (paths under
// src/ThunderEgg/) whose algorithm it restates; the operation order inside
// each loop follows the reference so that results agree to rounding.
//
// Parity of this restatement is pinned against the reference itself, compiled
// from its own sources (oracle/ref/, built into oracle/_ref/), by the tests in
// tests/test_oracle_pin.py and by the committed fixtures in tests/golden/.
//
// Data layout is ThunderEgg's Vector<D> (Vector.h:133-153): patches
// contiguous, each [component][z][y][x] with num_ghost padding per axis.

#include "te_gpu.h"
#include "te_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// faces (Face.h:41-584)
// ---------------------------------------------------------------------------
int num_faces(int D, int M) {
  if (D == 2) return 4;
  if (M == 1) return 12;
  return M == 0 ? 8 : 6;
}
int sum_of_faces(int D, int M) {
  if (D == 2) return M == 0 ? 0 : 4;
  return M == 0 ? 0 : (M == 1 ? 8 : 20);
}
int num_slots(int D) { return D == 2 ? 8 : 26; }
int face_opposite(int D, int M, int v) { return v ^ ((1 << (D - M)) - 1); }
// Face::getSides (Face.h:497-526): the D-M sides the face lies on, by axis
void face_sides(int D, int M, int v, int* axis, int* upper) {
  if (M == D - 1) {
    axis[0] = v >> 1;
    upper[0] = v & 1;
  } else if (M == 0) {
    for (int i = 0; i < D; i++) {
      axis[i] = i;
      upper[i] = (v >> i) & 1;
    }
  } else {  // D == 3, M == 1
    int not_axis = v >> 2, k = 0;
    for (int i = 0; i < 3; i++)
      if (i != not_axis) {
        axis[k] = i;
        upper[k] = (v >> k) & 1;
        k++;
      }
  }
}
void face_tangential(int D, int M, int v, int* tang) {
  int ax[3], up[3];
  face_sides(D, M, v, ax, up);
  int k = 0;
  for (int a = 0; a < D; a++) {
    bool on = false;
    for (int i = 0; i < D - M; i++) on |= ax[i] == a;
    if (!on) tang[k++] = a;
  }
}

// ---------------------------------------------------------------------------
// level = Domain<D> + PatchInfo tables
// ---------------------------------------------------------------------------
struct Level {
  int D = 2, n[3] = {1, 1, 1}, g = 1, P = 0;
  long s[3] = {1, 1, 1};  // spatial strides
  long cs = 1;            // component stride (cells of one padded component)
  std::vector<int> id, parent_id, orth_on_parent, child_ids, type, ids, orth, nloc;
  std::vector<double> starts, spacings;
  std::map<int, int> id2l;

  explicit Level(const te_level_desc* d) {
    D = d->dim;
    g = d->num_ghost;
    P = d->num_patches;
    for (int a = 0; a < 3; a++) n[a] = a < D ? d->ns[a] : 1;
    long st = 1;
    for (int a = 0; a < D; a++) {
      s[a] = st;
      st *= n[a] + 2 * g;
    }
    cs = st;
    int F = num_slots(D), C = 1 << D;
    id.assign(d->id, d->id + P);
    parent_id.assign(d->parent_id, d->parent_id + P);
    orth_on_parent.assign(d->orth_on_parent, d->orth_on_parent + P);
    child_ids.assign(d->child_ids, d->child_ids + (size_t)P * C);
    starts.assign(d->starts, d->starts + (size_t)P * D);
    spacings.assign(d->spacings, d->spacings + (size_t)P * D);
    type.assign(d->nbr_type, d->nbr_type + (size_t)P * F);
    ids.assign(d->nbr_ids, d->nbr_ids + (size_t)P * F * 4);
    orth.assign(d->nbr_orth, d->nbr_orth + (size_t)P * F);
    // Domain::indexPatchesLocal (Domain.h:94-110)
    for (int p = 0; p < P; p++) id2l[id[p]] = p;
    nloc.assign((size_t)P * F * 4, -1);
    for (size_t i = 0; i < nloc.size(); i++) {
      int t = type[i / 4];
      if (t < 0) continue;
      auto it = id2l.find(ids[i]);
      if (it != id2l.end()) nloc[i] = it->second;
    }
  }
  int F() const { return num_slots(D); }
  bool has(int p, int M, int v) const { return type[(size_t)p * F() + sum_of_faces(D, M) + v] >= 0; }
  int ntype(int p, int M, int v) const { return type[(size_t)p * F() + sum_of_faces(D, M) + v]; }
  int north(int p, int M, int v) const { return orth[(size_t)p * F() + sum_of_faces(D, M) + v]; }
  int nlocal(int p, int M, int v, int i) const {
    return nloc[((size_t)p * F() + sum_of_faces(D, M) + v) * 4 + i];
  }
  long pstride(int nc) const { return cs * nc; }
  size_t size(int nc) const { return (size_t)P * pstride(nc); }
  double h(int p, int a) const { return spacings[(size_t)p * D + a]; }
  bool has_any_nbr(int p) const {
    for (int i = 0; i < F(); i++)
      if (type[(size_t)p * F() + i] >= 0) return true;
    return false;
  }
  // linear index of cell (x,y,z) of component c in a patch
  long at(int x, int y, int z, int c) const {
    return (long)(x + g) * s[0] + (long)(y + g) * (D > 1 ? s[1] : 0) +
           (long)(z + g) * (D > 2 ? s[2] : 0) + (long)c * cs;
  }
};

// View over an M-dimensional face slice: M tangential coords then component
// (PatchView::getSliceOn / getGhostSliceOn, PatchView.h:100-240)
struct SV {
  double* b;
  long st[4];
  double& operator()(int c) const { return b[c * st[0]]; }
  double& operator()(int i, int c) const { return b[i * st[0] + c * st[1]]; }
  double& operator()(int i, int j, int c) const { return b[i * st[0] + j * st[1] + c * st[2]]; }
};

SV slice(const Level& L, double* patch, int M, int v, const int* off, bool ghost) {
  int ax[3], up[3], tang[3];
  face_sides(L.D, M, v, ax, up);
  face_tangential(L.D, M, v, tang);
  int coord[3] = {0, 0, 0};
  for (int i = 0; i < L.D - M; i++) {
    int a = ax[i];
    if (ghost)
      coord[a] = up[i] ? L.n[a] + off[i] : -1 - off[i];
    else
      coord[a] = up[i] ? L.n[a] - 1 - off[i] : off[i];
  }
  SV sv;
  sv.b = patch + L.at(coord[0], coord[1], coord[2], 0);
  for (int i = 0; i < M; i++) sv.st[i] = L.s[tang[i]];
  sv.st[M] = L.cs;
  return sv;
}
SV islice(const Level& L, double* patch, int M, int v, int o0 = 0, int o1 = 0, int o2 = 0) {
  int off[3] = {o0, o1, o2};
  return slice(L, patch, M, v, off, false);
}
SV gslice(const Level& L, double* patch, int M, int v, int o0 = 0, int o1 = 0, int o2 = 0) {
  int off[3] = {o0, o1, o2};
  return slice(L, patch, M, v, off, true);
}

// ---------------------------------------------------------------------------
// ghost filling (MPIGhostFiller.h:821-1092 and the three schemes)
// ---------------------------------------------------------------------------
struct Call {
  int local, nbr, M, face, type, orth;
};

// MPIGhostFiller::enumerateCalls (MPIGhostFiller.h:779-836): per M, patches in
// domain order, faces in value order; Fine neighbours give one call per orthant.
std::vector<Call> enumerate_calls(const Level& L, int M) {
  std::vector<Call> calls;
  for (int p = 0; p < L.P; p++)
    for (int f = 0; f < num_faces(L.D, M); f++) {
      if (!L.has(p, M, f)) continue;
      int t = L.ntype(p, M, f);
      if (t == TE_NBR_NORMAL)
        calls.push_back({p, L.nlocal(p, M, f, 0), M, f, t, -1});
      else if (t == TE_NBR_FINE)
        for (int i = 0; i < (1 << M); i++) calls.push_back({p, L.nlocal(p, M, f, i), M, f, t, i});
      else
        calls.push_back({p, L.nlocal(p, M, f, 0), M, f, t, L.north(p, M, f)});
    }
  return calls;
}

// dimensionalities filled for a GhostFillingType (switch fall-through,
// MPIGhostFiller.h:956-985): sides always, edges (3D) for Edges/Corners,
// corners for Corners.
std::vector<int> filled_dims(int D, int fill_type) {
  std::vector<int> ms;  // in processLocalFills order: D-1 down to 0
  ms.push_back(D - 1);
  if (D == 3 && fill_type >= TE_FILL_EDGES) ms.push_back(1);
  if (fill_type == TE_FILL_CORNERS) ms.push_back(0);
  return ms;
}

struct Scheme {
  virtual ~Scheme() {}
  virtual void local(const Level& L, int p, double* u, int nc, int fill_type) const = 0;
  virtual void nbr(const Level& L, const Call& c, double* lu, double* nu, int nc) const = 0;
};

// ---- BiLinearGhostFiller (BiLinearGhostFiller.cpp:40-388), 2D ----
struct BiLinear : Scheme {
  void nbr(const Level& L, const Call& cl, double* lu, double* nu, int nc) const override {
    int n = L.n[0];
    if (cl.M == 1) {
      int side = cl.face, opp = face_opposite(2, 1, side);
      SV ls = islice(L, lu, 1, side), ng = gslice(L, nu, 1, opp);
      int tang_axis = !(side >> 1);
      int tn = L.n[tang_axis];
      int offset = (cl.orth == 1) ? tn : 0;
      (void)n;
      for (int c = 0; c < nc; c++)
        for (int i = 0; i < tn; i++) {
          if (cl.type == TE_NBR_NORMAL)  // FillGhostForNormalNbr :40-48
            ng(i, c) = ls(i, c);
          else if (cl.type == TE_NBR_COARSE)  // FillGhostForCoarseNbr :61-76
            ng((i + offset) / 2, c) += 2.0 / 3.0 * ls(i, c);
          else  // FillGhostForFineNbr :90-105
            ng(i, c) += 2.0 / 3.0 * ls((i + offset) / 2, c);
        }
    } else {  // corners :147-210
      int corner = cl.face, opp = face_opposite(2, 0, corner);
      SV ls = islice(L, lu, 0, corner), ng = gslice(L, nu, 0, opp);
      for (int c = 0; c < nc; c++) {
        if (cl.type == TE_NBR_NORMAL)
          ng(c) = ls(c);
        else if (cl.type == TE_NBR_COARSE)
          ng(c) += 4.0 * ls(c) / 3.0;
        else
          ng(c) += 2.0 * ls(c) / 3.0;
      }
    }
  }
  void local(const Level& L, int p, double* u, int nc, int fill_type) const override {
    if (fill_type == TE_FILL_CORNERS)  // FillLocalGhostCellsOnCorners :294-313
      for (int corner = 0; corner < 4; corner++) {
        if (!L.has(p, 0, corner)) continue;
        int t = L.ntype(p, 0, corner);
        SV ls = islice(L, u, 0, corner), lg = gslice(L, u, 0, corner);
        for (int c = 0; c < nc; c++) {
          if (t == TE_NBR_COARSE)
            lg(c) += ls(c) / 3.0;
          else if (t == TE_NBR_FINE)
            lg(c) += -ls(c) / 3.0;
        }
      }
    for (int side = 0; side < 4; side++) {  // FillLocalGhostCellsOnSides :271-288
      if (!L.has(p, 1, side)) continue;
      int t = L.ntype(p, 1, side);
      SV ls = islice(L, u, 1, side), lg = gslice(L, u, 1, side);
      int tn = L.n[!(side >> 1)];
      if (t == TE_NBR_COARSE) {  // FillLocalGhostsForCoarseNbr :118-134
        int offset = L.north(p, 1, side) == 1 ? tn : 0;
        for (int c = 0; c < nc; c++)
          for (int i = 0; i < tn; i++) {
            lg(i, c) += 2.0 / 3.0 * ls(i, c);
            if ((i + offset) % 2 == 0)
              lg(i + 1, c) += -1.0 / 3.0 * ls(i, c);
            else
              lg(i - 1, c) += -1.0 / 3.0 * ls(i, c);
          }
      } else if (t == TE_NBR_FINE) {  // FillLocalGhostsForFineNbr :145-152
        for (int c = 0; c < nc; c++)
          for (int i = 0; i < tn; i++) lg(i, c) += -1.0 / 3.0 * ls(i, c);
      }
    }
  }
};

// ---- BiQuadraticGhostFiller (BiQuadraticGhostFiller.cpp:44-470), 2D ----
struct BiQuadratic : Scheme {
  void nbr(const Level& L, const Call& cl, double* lu, double* nu, int nc) const override {
    if (cl.M == 1) {
      int side = cl.face, opp = face_opposite(2, 1, side);
      SV slice0 = islice(L, lu, 1, side), inner = islice(L, lu, 1, side, 1);
      SV ghost = gslice(L, nu, 1, opp);
      int n = L.n[!(side >> 1)];
      for (int c = 0; c < nc; c++) {
        if (cl.type == TE_NBR_NORMAL) {  // FillGhostForNormalNbr :72-80
          for (int i = 0; i < n; i++) ghost(i, c) = slice0(i, c);
        } else if (cl.type == TE_NBR_COARSE) {
          if (cl.orth == 0)  // FillGhostForCoarseNbrLower :81-92
            for (int idx = 0; idx < n; idx++)
              ghost(idx / 2, c) += slice0(idx, c) / 3 + inner(idx, c) / 5;
          else  // FillGhostForCoarseNbrUpper :93-105
            for (int idx = 0; idx < n; idx++)
              ghost((idx + n) / 2, c) += slice0(idx, c) / 3 + inner(idx, c) / 5;
        } else {
          SV& s = slice0;
          if (cl.orth == 0) {  // FillGhostForFineNbrLower :106-126
            ghost(0, c) += 3 * s(0, c) / 4 - 3 * s(1, c) / 10 + s(2, c) / 12;
            ghost(1, c) += 7 * s(0, c) / 20 + 7 * s(1, c) / 30 - s(2, c) / 20;
            for (int idx = 2; idx < n; idx++) {
              if (idx % 2 == 0)
                ghost(idx, c) += s(idx / 2 - 1, c) / 12 + s(idx / 2, c) / 2 - s(idx / 2 + 1, c) / 20;
              else
                ghost(idx, c) += -s(idx / 2 - 1, c) / 20 + s(idx / 2, c) / 2 + s(idx / 2 + 1, c) / 12;
            }
          } else {  // FillGhostForFineNbrUpper :127-148
            for (int idx = 0; idx < n - 2; idx++) {
              if ((idx + n) % 2 == 0)
                ghost(idx, c) += s((idx + n) / 2 - 1, c) / 12 + s((idx + n) / 2, c) / 2 -
                                 s((idx + n) / 2 + 1, c) / 20;
              else
                ghost(idx, c) += -s((idx + n) / 2 - 1, c) / 20 + s((idx + n) / 2, c) / 2 +
                                 s((idx + n) / 2 + 1, c) / 12;
            }
            ghost(n - 2, c) += 7 * s(n - 1, c) / 20 + 7 * s(n - 2, c) / 30 - s(n - 3, c) / 20;
            ghost(n - 1, c) += 3 * s(n - 1, c) / 4 - 3 * s(n - 2, c) / 10 + s(n - 3, c) / 12;
          }
        }
      }
    } else {  // corners :150-205
      int corner = cl.face, opp = face_opposite(2, 0, corner);
      SV s = islice(L, lu, 0, corner), inner = islice(L, lu, 0, corner, 1, 1);
      SV ghost = gslice(L, nu, 0, opp);
      for (int c = 0; c < nc; c++) {
        if (cl.type == TE_NBR_NORMAL)
          ghost(c) = s(c);
        else if (cl.type == TE_NBR_COARSE)
          ghost(c) += 2 * s(c) / 3 + 2 * inner(c) / 5;
        else
          ghost(c) += 8 * s(c) / 15;
      }
    }
  }
  void local(const Level& L, int p, double* u, int nc, int fill_type) const override {
    if (fill_type == TE_FILL_CORNERS)  // FillLocalGhostCellsOnCorners :362-380
      for (int corner = 0; corner < 4; corner++) {
        if (!L.has(p, 0, corner)) continue;
        int t = L.ntype(p, 0, corner);
        SV s = islice(L, u, 0, corner), inner = islice(L, u, 0, corner, 1, 1);
        SV ghost = gslice(L, u, 0, corner);
        for (int c = 0; c < nc; c++) {
          if (t == TE_NBR_COARSE)
            ghost(c) += 2 * s(c) / 3 - inner(c) / 5;
          else if (t == TE_NBR_FINE)
            ghost(c) += -s(c) / 15;
        }
      }
    for (int side = 0; side < 4; side++) {  // FillLocalGhostCellsOnSides :341-360
      if (!L.has(p, 1, side)) continue;
      int t = L.ntype(p, 1, side);
      SV s = islice(L, u, 1, side), inner = islice(L, u, 1, side, 1);
      SV ghost = gslice(L, u, 1, side);
      int n = L.n[!(side >> 1)];
      for (int c = 0; c < nc; c++) {
        if (t == TE_NBR_COARSE) {  // FillGhostForLocalWithCoarseNbr :34-45
          for (int idx = 0; idx < n; idx++) ghost(idx, c) += 2 * s(idx, c) / 3 - inner(idx, c) / 5;
        } else if (t == TE_NBR_FINE) {  // FillGhostForLocalWithFineNbr :46-58
          ghost(0, c) += -s(0, c) / 10 + s(1, c) / 15 - s(2, c) / 30;
          for (int idx = 1; idx < n - 1; idx++) ghost(idx, c) += -s(idx - 1, c) / 30 - s(idx + 1, c) / 30;
          ghost(n - 1, c) += -s(n - 1, c) / 10 + s(n - 2, c) / 15 - s(n - 3, c) / 30;
        }
      }
    }
  }
};

// ---- TriLinearGhostFiller (TriLinearGhostFiller.cpp:28-590), 3D ----
struct TriLinear : Scheme {
  // getOffset (:28-44)
  static void get_offset(const Level& L, int side, int orth, int& oi, int& oj) {
    int axis = side >> 1, off[2] = {0, 0};
    for (int i = 0; i < axis; i++)
      if ((orth >> i) & 1) off[i] = L.n[i];
    for (int i = axis + 1; i < 3; i++)
      if ((orth >> (i - 1)) & 1) off[i - 1] = L.n[i];
    oi = off[0];
    oj = off[1];
  }
  void nbr(const Level& L, const Call& cl, double* lu, double* nu, int nc) const override {
    if (cl.M == 2) {
      int side = cl.face, opp = face_opposite(3, 2, side);
      SV ls = islice(L, lu, 2, side), ng = gslice(L, nu, 2, opp);
      int tang[2];
      face_tangential(3, 2, side, tang);
      int ni = L.n[tang[0]], nj = L.n[tang[1]];
      int oi = 0, oj = 0;
      if (cl.type != TE_NBR_NORMAL) get_offset(L, side, cl.orth, oi, oj);
      for (int c = 0; c < nc; c++)
        for (int j = 0; j < nj; j++)
          for (int i = 0; i < ni; i++) {
            if (cl.type == TE_NBR_NORMAL)  // :49-57
              ng(i, j, c) = ls(i, j, c);
            else if (cl.type == TE_NBR_COARSE)  // :58-73
              ng((i + oi) / 2, (j + oj) / 2, c) += 1.0 / 3.0 * ls(i, j, c);
            else  // :83-99
              ng(i, j, c) += 4.0 / 6.0 * ls((i + oi) / 2, (j + oj) / 2, c);
          }
    } else if (cl.M == 1) {
      int edge = cl.face, opp = face_opposite(3, 1, edge);
      SV ls = islice(L, lu, 1, edge), ng = gslice(L, nu, 1, opp);
      int n = L.n[edge >> 2];
      int offset = (cl.type != TE_NBR_NORMAL && cl.orth == 1) ? n : 0;
      for (int c = 0; c < nc; c++)
        for (int i = 0; i < n; i++) {
          if (cl.type == TE_NBR_NORMAL)  // :131-139
            ng(i, c) = ls(i, c);
          else if (cl.type == TE_NBR_COARSE)  // :140-155
            ng((i + offset) / 2, c) += 2.0 / 3.0 * ls(i, c);
          else  // :156-171
            ng(i, c) += 2.0 / 3.0 * ls((i + offset) / 2, c);
        }
    } else {
      int corner = cl.face, opp = face_opposite(3, 0, corner);
      SV ls = islice(L, lu, 0, corner), ng = gslice(L, nu, 0, opp);
      for (int c = 0; c < nc; c++) {
        if (cl.type == TE_NBR_NORMAL)
          ng(c) = ls(c);
        else if (cl.type == TE_NBR_COARSE)
          ng(c) += 4.0 * ls(c) / 3.0;
        else
          ng(c) += 2.0 * ls(c) / 3.0;
      }
    }
  }
  void local(const Level& L, int p, double* u, int nc, int fill_type) const override {
    if (fill_type == TE_FILL_CORNERS)  // :403-420
      for (int corner = 0; corner < 8; corner++) {
        if (!L.has(p, 0, corner)) continue;
        int t = L.ntype(p, 0, corner);
        SV ls = islice(L, u, 0, corner), lg = gslice(L, u, 0, corner);
        for (int c = 0; c < nc; c++) {
          if (t == TE_NBR_COARSE)
            lg(c) += ls(c) / 3.0;
          else if (t == TE_NBR_FINE)
            lg(c) += -ls(c) / 3.0;
        }
      }
    if (fill_type >= TE_FILL_EDGES)  // :385-402
      for (int edge = 0; edge < 12; edge++) {
        if (!L.has(p, 1, edge)) continue;
        int t = L.ntype(p, 1, edge);
        SV ls = islice(L, u, 1, edge), lg = gslice(L, u, 1, edge);
        int n = L.n[edge >> 2];
        if (t == TE_NBR_COARSE) {  // :172-195
          int offset = L.north(p, 1, edge) == 1 ? n : 0;
          for (int c = 0; c < nc; c++)
            for (int i = 0; i < n; i++) {
              lg(i, c) += 2.0 / 3.0 * ls(i, c);
              if ((i + offset) % 2 == 0)
                lg(i + 1, c) += -1.0 / 3.0 * ls(i, c);
              else
                lg(i - 1, c) += -1.0 / 3.0 * ls(i, c);
            }
        } else if (t == TE_NBR_FINE) {  // :196-203
          for (int c = 0; c < nc; c++)
            for (int i = 0; i < n; i++) lg(i, c) += -1.0 / 3.0 * ls(i, c);
        }
      }
    for (int side = 0; side < 6; side++) {  // :366-384
      if (!L.has(p, 2, side)) continue;
      int t = L.ntype(p, 2, side);
      SV ls = islice(L, u, 2, side), lg = gslice(L, u, 2, side);
      int tang[2];
      face_tangential(3, 2, side, tang);
      int ni = L.n[tang[0]], nj = L.n[tang[1]];
      if (t == TE_NBR_COARSE) {  // FillGhostCellsForLocalWithCoarseNbr :100-122
        int si, sj;
        get_offset(L, side, L.north(p, 2, side), si, sj);
        for (int c = 0; c < nc; c++)
          for (int j = 0; j < nj; j++) {
            int offj = (j + sj) % 2 == 0 ? (j + 1) : (j - 1);
            for (int i = 0; i < ni; i++) {
              lg(i, j, c) += 5.0 / 6.0 * ls(i, j, c);
              int offi = (i + si) % 2 == 0 ? (i + 1) : (i - 1);
              lg(i, j, c) -= 1.0 / 6.0 * ls(offi, j, c);
              lg(i, j, c) -= 1.0 / 6.0 * ls(i, offj, c);
              lg(i, j, c) -= 1.0 / 6.0 * ls(offi, offj, c);
            }
          }
      } else if (t == TE_NBR_FINE) {  // FillGhostCellsForLocalWithFineNbr :74-82
        for (int c = 0; c < nc; c++)
          for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) lg(i, j, c) -= 1.0 / 3.0 * ls(i, j, c);
      }
    }
  }
};

const Scheme& scheme_of(int s) {
  static BiLinear bl;
  static BiQuadratic bq;
  static TriLinear tl;
  if (s == TE_GHOST_BILINEAR) return bl;
  if (s == TE_GHOST_BIQUADRATIC) return bq;
  return tl;
}

// MPIGhostFiller::zeroGhostCellsOnAllFaces (MPIGhostFiller.h:905-928)
void zero_ghosts(const Level& L, int p, double* u, int nc, int M) {
  for (int f = 0; f < num_faces(L.D, M); f++) {
    if (!L.has(p, M, f)) continue;
    int k = L.D - M;
    int total = 1;
    for (int i = 0; i < k; i++) total *= L.g;
    for (int t = 0; t < total; t++) {
      int off[3] = {0, 0, 0}, r = t;
      for (int i = 0; i < k; i++) {
        off[i] = r % L.g;
        r /= L.g;
      }
      SV gs = slice(L, u, M, f, off, true);
      int tang[3];
      face_tangential(L.D, M, f, tang);
      int n0 = M > 0 ? L.n[tang[0]] : 1, n1 = M > 1 ? L.n[tang[1]] : 1;
      for (int c = 0; c < nc; c++)
        for (int j = 0; j < n1; j++)
          for (int i = 0; i < n0; i++) {
            if (M == 0)
              gs(c) = 0;
            else if (M == 1)
              gs(i, c) = 0;
            else
              gs(i, j, c) = 0;
          }
    }
  }
}

struct GhostFiller {
  const Level& L;
  int scheme, fill_type;
  std::vector<std::vector<Call>> calls;  // in processLocalFills order
  GhostFiller(const Level& L, int scheme, int fill_type) : L(L), scheme(scheme), fill_type(fill_type) {
    for (int M : filled_dims(L.D, fill_type)) calls.push_back(enumerate_calls(L, M));
  }
  // MPIGhostFiller::fillGhost (MPIGhostFiller.h:1055-1092), single rank
  void fill(double* u, int nc) const {
    long ps = L.pstride(nc);
    for (int p = 0; p < L.P; p++) {  // zeroGhostCells :929-947
      double* up = u + p * ps;
      if (fill_type == TE_FILL_CORNERS) zero_ghosts(L, p, up, nc, 0);
      if (L.D == 3 && fill_type >= TE_FILL_EDGES) zero_ghosts(L, p, up, nc, 1);
      zero_ghosts(L, p, up, nc, L.D - 1);
    }
    const Scheme& sc = scheme_of(scheme);
    for (int p = 0; p < L.P; p++) sc.local(L, p, u + p * ps, nc, fill_type);
    for (auto& list : calls)
      for (auto& c : list) sc.nbr(L, c, u + c.local * ps, u + c.nbr * ps, nc);
  }
};

// ---------------------------------------------------------------------------
// vector algebra (Vector.h:391-611) over "interior" cells of P patches
// ---------------------------------------------------------------------------
template <class Fn>
void for_interior(const Level& L, int P, int nc, Fn fn) {
  long ps = L.pstride(nc);
  for (int p = 0; p < P; p++)
    for (int c = 0; c < nc; c++)
      for (int z = 0; z < L.n[2]; z++)
        for (int y = 0; y < L.n[1]; y++)
          for (int x = 0; x < L.n[0]; x++) fn(p * ps + L.at(x, y, z, c));
}

// ---------------------------------------------------------------------------
// Poisson / VarPoisson star operators
// ---------------------------------------------------------------------------
struct Op {
  const Level& L;
  GhostFiller gf;
  int kind;  // 0 Poisson, 1 VarPoisson
  bool neumann;
  std::vector<double> coeffs;
  Op(const Level& L, int scheme, int fill_type, int kind, bool neumann, const double* c)
      : L(L), gf(L, scheme, fill_type), kind(kind), neumann(neumann) {
    if (kind == 1) {
      coeffs.assign(c, c + L.size(1));
      gf.fill(coeffs.data(), 1);  // VarPoisson ctor fills coefficient ghosts (:61-71)
    }
  }
  // StarPatchOperator::enforceBoundaryConditions (Poisson :106-135, VarPoisson :115-133)
  void enforce_bc(int p, double* u, int nc, bool internal) const {
    for (int axis = 0; axis < L.D; axis++)
      for (int up = 0; up < 2; up++) {
        int side = 2 * axis + up;
        bool has = L.has(p, L.D - 1, side);
        if (internal != has) continue;
        SV g = gslice(L, u, L.D - 1, side), m = islice(L, u, L.D - 1, side);
        int tang[2];
        face_tangential(L.D, L.D - 1, side, tang);
        int n0 = L.n[tang[0]], n1 = L.D == 3 ? L.n[tang[1]] : 1;
        bool copy = (!internal && neumann && kind == 0);
        for (int c = 0; c < nc; c++)
          for (int j = 0; j < n1; j++)
            for (int i = 0; i < n0; i++) {
              if (L.D == 2)
                g(i, c) = copy ? m(i, c) : -m(i, c);
              else
                g(i, j, c) = copy ? m(i, j, c) : -m(i, j, c);
            }
      }
  }
  // applySinglePatch (Poisson/StarPatchOperator.h:75-101; VarPoisson :78-110)
  void apply_patch(int p, double* u, double* f, int nc, bool internal) const {
    if (internal) enforce_bc(p, u, nc, true);
    enforce_bc(p, u, nc, false);
    const double* cp = kind == 1 ? coeffs.data() + p * L.pstride(1) : nullptr;
    for (int axis = 0; axis < L.D; axis++) {
      double h2 = L.h(p, axis) * L.h(p, axis);
      long st = L.s[axis];
      for (int c = 0; c < nc; c++)
        for (int z = 0; z < L.n[2]; z++)
          for (int y = 0; y < L.n[1]; y++)
            for (int x = 0; x < L.n[0]; x++) {
              long i = L.at(x, y, z, c);
              double lower = u[i - st], mid = u[i], upper = u[i + st];
              double add = axis == 0 ? 0 : 1;
              if (kind == 0) {
                f[i] = add * f[i] + (upper - 2 * mid + lower) / h2;
              } else {
                long ci = L.at(x, y, z, 0);
                double cl = cp[ci - st], cm = cp[ci], cu = cp[ci + st];
                f[i] = add * f[i] + ((cu + cm) * (upper - mid) - (cl + cm) * (mid - lower)) / (2 * h2);
              }
            }
    }
  }
  // PatchOperator::apply (PatchOperator.h:126-143)
  void apply(double* u, double* f, int nc) const {
    std::fill(f, f + L.size(nc), 0.0);
    gf.fill(u, nc);
    long ps = L.pstride(nc);
    for (int p = 0; p < L.P; p++) apply_patch(p, u + p * ps, f + p * ps, nc, false);
  }
  // modifyRHSForInternalBoundaryConditions (Poisson :145-164 (165-180); VarPoisson :134-153)
  void modify_rhs(int p, const double* u, double* f, int nc) const {
    const double* cp = kind == 1 ? coeffs.data() + p * L.pstride(1) : nullptr;
    for (int side = 0; side < 2 * L.D; side++) {
      if (!L.has(p, L.D - 1, side)) continue;
      double h2 = std::pow(L.h(p, side >> 1), 2);
      SV fi = islice(L, f, L.D - 1, side);
      SV ug = islice(L, const_cast<double*>(u), L.D - 1, side, -1);
      SV ui = islice(L, const_cast<double*>(u), L.D - 1, side);
      SV cg{}, ci{};
      if (kind == 1) {
        cg = islice(L, const_cast<double*>(cp), L.D - 1, side, -1);
        ci = islice(L, const_cast<double*>(cp), L.D - 1, side);
      }
      int tang[2];
      face_tangential(L.D, L.D - 1, side, tang);
      int n0 = L.n[tang[0]], n1 = L.D == 3 ? L.n[tang[1]] : 1;
      for (int c = 0; c < nc; c++)
        for (int j = 0; j < n1; j++)
          for (int i = 0; i < n0; i++) {
            double *fv, uv, gv, civ = 0, cgv = 0;
            if (L.D == 2) {
              fv = &fi(i, c);
              gv = ug(i, c);
              uv = ui(i, c);
              if (kind == 1) {
                civ = ci(i, 0);
                cgv = cg(i, 0);
              }
            } else {
              fv = &fi(i, j, c);
              gv = ug(i, j, c);
              uv = ui(i, j, c);
              if (kind == 1) {
                civ = ci(i, j, 0);
                cgv = cg(i, j, 0);
              }
            }
            if (kind == 0)
              *fv -= (gv + uv) / h2;
            else
              *fv -= (gv + uv) * (civ + cgv) / (2 * h2);
          }
    }
  }
};

// ---------------------------------------------------------------------------
// BiCGStab (Iterative/BiCGStab.h:111-203) over a generic vector space
// ---------------------------------------------------------------------------
struct Space {
  const Level& L;
  int P, nc;
  size_t size() const { return (size_t)P * L.pstride(nc); }
  std::vector<double> zero() const { return std::vector<double>(size(), 0.0); }
  template <class Fn>
  void each(Fn fn) const { for_interior(L, P, nc, fn); }
  double dot(const double* a, const double* b) const {
    double s = 0;
    each([&](long i) { s += a[i] * b[i]; });
    return s;
  }
  double norm(const double* a) const { return std::sqrt(dot(a, a)); }
};
using ApplyFn = std::function<void(double* x, double* b)>;

int bicgstab(const Space& V, const ApplyFn& A, double* x, const double* b, const ApplyFn* Mr,
             double tol, int max_it, double* final_res, bool* breakdown, bool precond_exit = false) {
  *breakdown = false;
  std::vector<double> resid = V.zero(), ms, mp;
  if (Mr) {
    ms = V.zero();
    mp = V.zero();
  }
  A(x, resid.data());
  V.each([&](long i) { resid[i] = resid[i] * -1 + b[i]; });  // scaleThenAdd(-1, b)
  double r0 = V.norm(b);
  std::vector<double> rhat = resid, p = resid, ap = V.zero(), as = V.zero(), s = V.zero();
  double rho = V.dot(rhat.data(), resid.data());
  int its = 0;
  double residual = V.norm(resid.data()) / r0;
  if (final_res) *final_res = residual;
  if (r0 == 0) return its;
  while (residual > tol && its < max_it) {
    if (rho == 0) {
      *breakdown = true;
      return its;
    }
    if (Mr) {
      (*Mr)(p.data(), mp.data());
      A(mp.data(), ap.data());
    } else {
      A(p.data(), ap.data());
    }
    double alpha = rho / V.dot(rhat.data(), ap.data());
    V.each([&](long i) { s[i] = resid[i]; });
    V.each([&](long i) { s[i] += ap[i] * -alpha; });
    if (V.norm(s.data()) / r0 <= tol) {
      // BiCGStab.h:162-168 adds alpha * p; with precond_exit the right-preconditioned
      // update alpha * M p (the GPU's TE_BICGSTAB_PRECONDITIONED_EXIT)
      if (Mr && precond_exit)
        V.each([&](long i) { x[i] += mp[i] * alpha; });
      else
        V.each([&](long i) { x[i] += p[i] * alpha; });
      break;
    }
    if (Mr) {
      (*Mr)(s.data(), ms.data());
      A(ms.data(), as.data());
    } else {
      A(s.data(), as.data());
    }
    double omega = V.dot(as.data(), s.data()) / V.dot(as.data(), as.data());
    if (Mr)
      V.each([&](long i) { x[i] += mp[i] * alpha + ms[i] * omega; });
    else
      V.each([&](long i) { x[i] += p[i] * alpha + s[i] * omega; });
    V.each([&](long i) { resid[i] += ap[i] * -alpha + as[i] * -omega; });
    double rho_new = V.dot(resid.data(), rhat.data());
    double beta = rho_new * alpha / (rho * omega);
    V.each([&](long i) { p[i] += ap[i] * -omega; });
    V.each([&](long i) { p[i] = p[i] * beta + resid[i]; });
    its++;
    rho = rho_new;
    residual = V.norm(resid.data()) / r0;
    if (final_res) *final_res = residual;
  }
  return its;
}

// ---------------------------------------------------------------------------
// patch solvers
// ---------------------------------------------------------------------------
enum DftType { DCT_II, DCT_III, DCT_IV, DST_II, DST_III, DST_IV };

struct Smoother {
  virtual ~Smoother() {}
  virtual void solve_patch(int p, const double* f, double* u, int nc) const = 0;
  const Op* op = nullptr;
  // PatchSolver::smooth (PatchSolver.h:142-170)
  void smooth(const double* f, double* u, int nc) const {
    op->gf.fill(u, nc);
    long ps = op->L.pstride(nc);
    for (int p = 0; p < op->L.P; p++) solve_patch(p, f + p * ps, u + p * ps, nc);
  }
  // PatchSolver::apply (PatchSolver.h:107-134)
  void apply(const double* f, double* u, int nc) const {
    std::fill(u, u + op->L.size(nc), 0.0);
    long ps = op->L.pstride(nc);
    for (int p = 0; p < op->L.P; p++) solve_patch(p, f + p * ps, u + p * ps, nc);
  }
};

// Poisson::DFTPatchSolver (Poisson/DFTPatchSolver.h:47-451)
struct DFTSolver : Smoother {
  int neumann;  // bitset over sides
  std::map<std::pair<int, int>, std::vector<double>> mats;
  struct Plan {
    int fwd[3], inv[3];
    std::vector<double> eig;  // n0*n1*n2 (no ghosts)
  };
  std::map<std::pair<unsigned long, double>, Plan> plans;

  bool neu_side(int p, int side) const { return !op->L.has(p, op->L.D - 1, side) && ((neumann >> side) & 1); }
  std::pair<unsigned long, double> key(int p) const {
    unsigned long m = 0;
    for (int s = 0; s < 2 * op->L.D; s++)
      if (neu_side(p, s)) m |= 1ul << s;
    return {m, op->L.h(p, 0)};
  }
  // getTransformArray (:131-196): matrix[i*n+j]
  const std::vector<double>& matrix(int type, int n) {
    auto k = std::make_pair(type, n);
    auto it = mats.find(k);
    if (it != mats.end()) return it->second;
    std::vector<double> m(n * n);
    switch (type) {
      case DCT_II:
        for (int j = 0; j < n; j++)
          for (int i = 0; i < n; i++) m[i * n + j] = std::cos(M_PI / n * (i * (j + 0.5)));
        break;
      case DCT_III:
        for (int i = 0; i < n; i++) m[i * n] = 0.5;
        for (int j = 1; j < n; j++)
          for (int i = 0; i < n; i++) m[i * n + j] = std::cos(M_PI / n * ((i + 0.5) * j));
        break;
      case DCT_IV:
        for (int j = 0; j < n; j++)
          for (int i = 0; i < n; i++) m[i * n + j] = std::cos(M_PI / n * ((i + 0.5) * (j + 0.5)));
        break;
      case DST_II:
        for (int i = 0; i < n; i++)
          for (int j = 0; j < n; j++) m[i * n + j] = std::sin(M_PI / n * ((i + 1) * (j + 0.5)));
        break;
      case DST_III:
        for (int i = 0; i < n; i += 2) m[i * n + n - 1] = 0.5;
        for (int i = 1; i < n; i += 2) m[i * n + n - 1] = -0.5;
        for (int i = 0; i < n; i++)
          for (int j = 0; j < n - 1; j++) m[i * n + j] = std::sin(M_PI / n * ((i + 0.5) * (j + 1)));
        break;
      case DST_IV:
        for (int j = 0; j < n; j++)
          for (int i = 0; i < n; i++) m[i * n + j] = std::sin(M_PI / n * ((i + 0.5) * (j + 0.5)));
        break;
    }
    return mats[k] = m;
  }
  DFTSolver(const Op* o, int neumann_mask) : neumann(neumann_mask) {
    op = o;
    const Level& L = op->L;
    for (int p = 0; p < L.P; p++) {  // addPatch (:362-369): first patch of each key
      auto k = key(p);
      if (plans.count(k)) continue;
      Plan pl;
      for (int a = 0; a < L.D; a++) {  // getTransformsForPatch (:272-313)
        bool lo = neu_side(p, 2 * a), hi = neu_side(p, 2 * a + 1);
        pl.fwd[a] = (lo && hi) ? DCT_II : lo ? DCT_IV : hi ? DST_IV : DST_II;
        pl.inv[a] = (lo && hi) ? DCT_III : lo ? DCT_IV : hi ? DST_IV : DST_III;
        matrix(pl.fwd[a], L.n[a]);
        matrix(pl.inv[a], L.n[a]);
      }
      // getEigenValues (:320-361)
      int tot = L.n[0] * L.n[1] * L.n[2];
      pl.eig.assign(tot, 0.0);
      for (int a = 0; a < L.D; a++) {
        int n = L.n[a];
        double h = L.h(p, a);
        bool lo = neu_side(p, 2 * a), hi = neu_side(p, 2 * a + 1);
        for (int xi = 0; xi < n; xi++) {
          double val;
          if (lo && hi)
            val = 4 / (h * h) * std::pow(std::sin(xi * M_PI / (2 * n)), 2);
          else if (lo || hi)
            val = 4 / (h * h) * std::pow(std::sin((xi + 0.5) * M_PI / (2 * n)), 2);
          else
            val = 4 / (h * h) * std::pow(std::sin((xi + 1) * M_PI / (2 * n)), 2);
          for (int i = 0; i < tot; i++) {
            int cidx[3] = {i % L.n[0], (i / L.n[0]) % L.n[1], i / (L.n[0] * L.n[1])};
            if (cidx[a] == xi) pl.eig[i] -= val;
          }
        }
      }
      plans[k] = pl;
    }
  }
  // y_line = M x_line with dgemv_('T', n, n, 1, M, n, x, stride, 0, y, stride), y[i] = sum_j M[i*n+j] x[j]
  static void line(const double* M, int n, const double* x, long xs, double* y, long ys) {
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = 0; j < n; j++) s += M[(long)i * n + j] * x[j * xs];
      y[i * ys] = s;
    }
  }
  // executePlan (:205-265) on ghost-free arrays [c][z][y][x] (PatchArray<D>(ns,1,0))
  // "in" may be overwritten; result in "out"
  void execute(const int* types, double* in, double* out, double* tmp2d, int nc, bool out_is_patch,
               double* u_patch) const {
    const Level& L = op->L;
    int D = L.D;
    long fs[3] = {1, L.n[0], (long)L.n[0] * L.n[1]};
    long fcs = (long)L.n[0] * L.n[1] * L.n[2];
    // buffer descriptors: 0 = in, 1 = out, 2 = local_tmp; the "out" buffer is
    // either a ghost-free array or the u patch (with ghosts).
    auto base = [&](int which) -> double* { return which == 0 ? in : which == 2 ? tmp2d : (out_is_patch ? u_patch : out); };
    auto stride = [&](int which, int a) -> long { return (which == 1 && out_is_patch) ? L.s[a] : fs[a]; };
    auto cstride = [&](int which) -> long { return (which == 1 && out_is_patch) ? L.cs : fcs; };
    auto idx = [&](int which, int x, int y, int z, int c) -> long {
      if (which == 1 && out_is_patch) return L.at(x, y, z, c);
      return x * fs[0] + y * fs[1] + z * fs[2] + c * fcs;
    };
    int prev = 0;
    for (int axis = 0; axis < D; axis++) {
      int n = L.n[axis];
      int nw;
      if (D % 2) {
        nw = (axis % 2) ? 0 : 1;
      } else {
        if (axis == D - 1)
          nw = 1;
        else if (axis == D - 2)
          nw = 2;
        else if (axis % 2)
          nw = 0;
        else
          nw = 1;
      }
      const std::vector<double>& M = mats.at({types[axis], n});
      int end[3] = {L.n[0], L.n[1], L.n[2]};
      end[axis] = 1;
      (void)cstride;
      for (int c = 0; c < nc; c++)
        for (int z = 0; z < end[2]; z++)
          for (int y = 0; y < end[1]; y++)
            for (int x = 0; x < end[0]; x++)
              line(M.data(), n, base(prev) + idx(prev, x, y, z, c), stride(prev, axis),
                   base(nw) + idx(nw, x, y, z, c), stride(nw, axis));
      prev = nw;
    }
  }
  // solveSinglePatch (:420-450)
  void solve_patch(int p, const double* f, double* u, int nc) const override {
    const Level& L = op->L;
    long tot = (long)L.n[0] * L.n[1] * L.n[2];
    std::vector<double> fcopy(tot * nc), tmp(tot * nc), ltmp(tot * nc);
    // f_copy as a ghosted patch so modifyRHS can use the same slices
    std::vector<double> fpatch(L.pstride(nc), 0.0);
    for (int c = 0; c < nc; c++)
      for (int z = 0; z < L.n[2]; z++)
        for (int y = 0; y < L.n[1]; y++)
          for (int x = 0; x < L.n[0]; x++) fpatch[L.at(x, y, z, c)] = f[L.at(x, y, z, c)];
    op->modify_rhs(p, u, fpatch.data(), nc);
    for (int c = 0; c < nc; c++)
      for (int z = 0; z < L.n[2]; z++)
        for (int y = 0; y < L.n[1]; y++)
          for (int x = 0; x < L.n[0]; x++)
            fcopy[x + y * L.n[0] + z * L.n[0] * L.n[1] + c * tot] = fpatch[L.at(x, y, z, c)];
    const Plan& pl = plans.at(key(p));
    execute(pl.fwd, fcopy.data(), tmp.data(), ltmp.data(), nc, false, nullptr);
    for (int c = 0; c < nc; c++)
      for (long i = 0; i < tot; i++) tmp[i + c * tot] /= pl.eig[i];
    if (neumann == (1 << (2 * L.D)) - 1 && !L.has_any_nbr(p)) tmp[0] = 0;
    execute(pl.inv, tmp.data(), nullptr, ltmp.data(), nc, true, u);
    double scale = 1;
    for (int a = 0; a < L.D; a++) scale *= 2.0 / L.n[a];
    for (int c = 0; c < nc; c++)
      for (int z = 0; z < L.n[2]; z++)
        for (int y = 0; y < L.n[1]; y++)
          for (int x = 0; x < L.n[0]; x++) u[L.at(x, y, z, c)] *= scale;
  }
};

// Iterative::PatchSolver with inner BiCGStab (Iterative/PatchSolver.h:121-175)
struct BiCGStabPatchSolver : Smoother {
  double tol;
  int max_it;
  bool cont;
  mutable long inner_iterations = 0;
  BiCGStabPatchSolver(const Op* o, double tol, int max_it, bool cont) : tol(tol), max_it(max_it), cont(cont) {
    op = o;
  }
  void solve_patch(int p, const double* f, double* u, int nc) const override {
    const Level& L = op->L;
    Space V{L, 1, nc};
    std::vector<double> fcopy = V.zero();
    V.each([&](long i) { fcopy[i] = f[i]; });
    op->modify_rhs(p, u, fcopy.data(), nc);
    ApplyFn A = [&](double* x, double* b) { op->apply_patch(p, x, b, nc, true); };
    bool bd;
    double fr;
    int its = bicgstab(V, A, u, fcopy.data(), nullptr, tol, max_it, &fr, &bd);
    inner_iterations += its;
    if (bd && !cont) throw std::runtime_error("BiCGStab broke down");
  }
};

// ---------------------------------------------------------------------------
// GMG transfers
// ---------------------------------------------------------------------------
// InterLevelComm parent map (InterLevelComm.h:125-160): fine patch -> parent local index
std::vector<int> parent_map(const Level& fine, const Level& coarse) {
  std::vector<int> m(fine.P, -1);
  for (int p = 0; p < fine.P; p++) {
    auto it = coarse.id2l.find(fine.parent_id[p]);
    m[p] = it == coarse.id2l.end() ? -1 : it->second;
  }
  return m;
}

// LinearRestrictor (GMG/LinearRestrictor.h:49-191) via MPIRestrictor::restrict (:55-83)
void restrict_vec(const Level& F, const Level& C, bool extrapolate, const double* fine, double* coarse,
                  int nc) {
  std::fill(coarse, coarse + C.size(nc), 0.0);
  auto pm = parent_map(F, C);
  long fps = F.pstride(nc), cps = C.pstride(nc);
  int D = F.D;
  for (int p = 0; p < F.P; p++) {
    const double* fv = fine + p * fps;
    double* cv = coarse + (long)pm[p] * cps;
    int orth = F.orth_on_parent[p];
    if (orth >= 0) {  // restrictToCoarserParent (:101-128)
      int st[3] = {0, 0, 0};
      for (int a = 0; a < D; a++) st[a] = ((orth >> a) & 1) ? C.n[a] : 0;
      for (int c = 0; c < nc; c++)
        for (int z = 0; z < F.n[2]; z++)
          for (int y = 0; y < F.n[1]; y++)
            for (int x = 0; x < F.n[0]; x++)
              cv[C.at((x + st[0]) / 2, D > 1 ? (y + st[1]) / 2 : 0, D > 2 ? (z + st[2]) / 2 : 0, c)] +=
                  fv[F.at(x, y, z, c)] / (1 << D);
      if (extrapolate) {  // extrapolateBoundaries (:49-100)
        for (int a = 0; a < D; a++) {
          int side = 2 * a + ((orth >> a) & 1);
          SV fg = islice(F, const_cast<double*>(fv), D - 1, side, -1);
          SV fi = islice(F, const_cast<double*>(fv), D - 1, side, 0);
          SV cg = islice(C, cv, D - 1, side, -1);
          int tang[2];
          face_tangential(D, D - 1, side, tang);
          int n0 = F.n[tang[0]], n1 = D == 3 ? F.n[tang[1]] : 1;
          for (int c = 0; c < nc; c++)
            for (int j = 0; j < n1; j++)
              for (int i = 0; i < n0; i++) {
                int ci0 = (i + st[tang[0]]) / 2;
                if (D == 2)
                  cg(ci0, c) += (3 * fg(i, c) - fi(i, c)) / (1 << D);
                else {
                  int ci1 = (j + st[tang[1]]) / 2;
                  cg(ci0, ci1, c) += (3 * fg(i, j, c) - fi(i, j, c)) / (1 << D);
                }
              }
        }
        int corner = orth;
        if (!F.has(p, 0, corner)) {
          SV fg = islice(F, const_cast<double*>(fv), 0, corner, -1, -1, -1);
          SV fi = islice(F, const_cast<double*>(fv), 0, corner, 0, 0, 0);
          SV cg = islice(C, cv, 0, corner, -1, -1, -1);
          for (int c = 0; c < nc; c++) cg(c) += (3 * fg(c) - fi(c));
        }
      }
    } else {  // copyToParent (:129-147)
      if (extrapolate) {
        for (long i = 0; i < fps; i++) cv[i] += fv[i];
      } else {
        for (int c = 0; c < nc; c++)
          for (int z = 0; z < F.n[2]; z++)
            for (int y = 0; y < F.n[1]; y++)
              for (int x = 0; x < F.n[0]; x++) cv[F.at(x, y, z, c)] += fv[F.at(x, y, z, c)];
      }
    }
  }
}

// DirectInterpolator (GMG/DirectInterpolator.h:60-91)
void interpolate_vec(const Level& C, const Level& F, const double* coarse, double* fine, int nc) {
  auto pm = parent_map(F, C);
  long fps = F.pstride(nc), cps = C.pstride(nc);
  int D = F.D;
  for (int p = 0; p < F.P; p++) {
    double* fv = fine + p * fps;
    const double* cv = coarse + (long)pm[p] * cps;
    int orth = F.orth_on_parent[p];
    int st[3] = {0, 0, 0};
    if (orth >= 0)
      for (int a = 0; a < D; a++) st[a] = ((orth >> a) & 1) ? C.n[a] : 0;
    for (int c = 0; c < nc; c++)
      for (int z = 0; z < F.n[2]; z++)
        for (int y = 0; y < F.n[1]; y++)
          for (int x = 0; x < F.n[0]; x++) {
            if (orth >= 0)
              fv[F.at(x, y, z, c)] +=
                  cv[C.at((x + st[0]) / 2, D > 1 ? (y + st[1]) / 2 : 0, D > 2 ? (z + st[2]) / 2 : 0, c)];
            else
              fv[F.at(x, y, z, c)] += cv[F.at(x, y, z, c)];
          }
  }
}

// ---------------------------------------------------------------------------
// GMG cycles (GMG/Cycle.h:57-98; VCycle.h:46-70, WCycle.h:50-84,
// FMGCycle.h:43-104) and the outer solve
// ---------------------------------------------------------------------------
struct Hierarchy {
  std::vector<Level> levels;
  std::vector<Op*> ops;
  std::vector<Smoother*> smoothers;
  int pre = 1, post = 1, coarse_sweeps = 1, mid = 1;
  int type = 0;  // 0 V, 1 W, 2 FMG
  bool extrapolate = false;
  ~Hierarchy() {
    for (auto* o : ops) delete o;
    for (auto* s : smoothers) delete s;
  }
  // Cycle::restrict (:57-65): the restriction of r = f - A u
  std::vector<double> restrict_residual(int k, const double* f, double* u, int nc) const {
    const Level& L = levels[k];
    std::vector<double> r(L.size(nc), 0.0);
    ops[k]->apply(u, r.data(), nc);
    for_interior(L, L.P, nc, [&](long i) { r[i] = r[i] * -1 + f[i]; });
    const Level& C = levels[k + 1];
    std::vector<double> cf(C.size(nc));
    restrict_vec(L, C, extrapolate, r.data(), cf.data(), nc);
    return cf;
  }
  void sweeps(int k, const double* f, double* u, int nc, int n) const {
    for (int i = 0; i < n; i++) smoothers[k]->smooth(f, u, nc);
  }
  // VCycle::visit, WCycle::visit, FMGCycle::visit.  W and FMG smooth mid_sweeps
  // times after the first coarse correction and visit the coarser level a
  // second time from that level's first result (the coarse vector is not
  // zeroed again, as in the reference); FMG's second visit is its v_visit.
  void visit(int k, const double* f, double* u, int nc) const {
    if (k + 1 == (int)levels.size()) {
      sweeps(k, f, u, nc, coarse_sweeps);
      return;
    }
    sweeps(k, f, u, nc, pre);
    std::vector<double> cf = restrict_residual(k, f, u, nc);
    const Level& C = levels[k + 1];
    const Level& L = levels[k];
    std::vector<double> cu(C.size(nc), 0.0);
    visit(k + 1, cf.data(), cu.data(), nc);
    interpolate_vec(C, L, cu.data(), u, nc);
    if (type != 0) {
      sweeps(k, f, u, nc, mid);
      cf = restrict_residual(k, f, u, nc);
      if (type == 1)
        visit(k + 1, cf.data(), cu.data(), nc);
      else
        v_visit(k + 1, cf.data(), cu.data(), nc);
      interpolate_vec(C, L, cu.data(), u, nc);
    }
    sweeps(k, f, u, nc, post);
  }
  // FMGCycle::v_visit (:43-66): one pre/post-smoothed pass whose coarser visit is visit()
  void v_visit(int k, const double* f, double* u, int nc) const {
    if (k + 1 == (int)levels.size()) {
      sweeps(k, f, u, nc, coarse_sweeps);
      return;
    }
    sweeps(k, f, u, nc, pre);
    std::vector<double> cf = restrict_residual(k, f, u, nc);
    const Level& C = levels[k + 1];
    std::vector<double> cu(C.size(nc), 0.0);
    visit(k + 1, cf.data(), cu.data(), nc);
    interpolate_vec(C, levels[k], cu.data(), u, nc);
    sweeps(k, f, u, nc, post);
  }
  void apply(const double* f, double* u, int nc) const {
    std::fill(u, u + levels[0].size(nc), 0.0);
    visit(0, f, u, nc);
  }
};

thread_local std::string g_err;

int guard(const std::function<void()>& fn) {
  try {
    fn();
    return TE_OK;
  } catch (const std::exception& e) {
    g_err = e.what();
    return TE_ERR_INVALID;
  }
}

}  // namespace

// ===========================================================================
// C API of the oracle (host pointers).  Signatures mirror include/te_gpu.h.
// ===========================================================================
extern "C" {

const char* teo_last_error(void) { return g_err.c_str(); }

int teo_ghost_fill(const te_level_desc* d, int scheme, int fill_type, int nc, double* u) {
  return guard([&] {
    Level L(d);
    GhostFiller gf(L, scheme, fill_type);
    gf.fill(u, nc);
  });
}

int teo_ghost_num_calls(const te_level_desc* d, int fill_type) {
  Level L(d);
  int n = 0;
  for (int M : filled_dims(L.D, fill_type)) n += (int)enumerate_calls(L, M).size();
  return n;
}

int teo_ghost_calls(const te_level_desc* d, int fill_type, int* rows6) {
  return guard([&] {
    Level L(d);
    int k = 0;
    for (int M : filled_dims(L.D, fill_type))
      for (auto& c : enumerate_calls(L, M)) {
        int r[6] = {c.local, c.nbr, c.M, c.face, c.type, c.orth};
        std::memcpy(rows6 + 6 * k++, r, sizeof r);
      }
  });
}

int teo_operator_apply(const te_level_desc* d, int scheme, int fill_type, int kind, int neumann,
                       const double* coeffs, int nc, double* u, double* f) {
  return guard([&] {
    Level L(d);
    Op op(L, scheme, fill_type, kind, neumann != 0, coeffs);
    op.apply(u, f, nc);
  });
}

int teo_modify_rhs(const te_level_desc* d, int scheme, int fill_type, int kind, const double* coeffs,
                   int nc, const double* u, double* f) {
  return guard([&] {
    Level L(d);
    Op op(L, scheme, fill_type, kind, false, coeffs);
    long ps = L.pstride(nc);
    for (int p = 0; p < L.P; p++) op.modify_rhs(p, u + p * ps, f + p * ps, nc);
  });
}

// Right-hand-side boundary helpers: Poisson::StarPatchOperator::addDrichletBCToRHS
// (Poisson/StarPatchOperator.h:187-204) and addNeumannBCToRHS (:212-242),
// VarPoisson::StarPatchOperator::addDrichletBCToRHS (VarPoisson/StarPatchOperator.h:194-219).
// Every side without a neighbour, in side order, adds to the interior cells next to it a
// term of the boundary data at the point DomainTools::GetRealCoordBound gives
// (DomainTools.h:179-210): the side's own coordinate on the boundary, the cell centre in
// the other directions.  kind 0 Poisson, 1 VarPoisson (hfun = coefficient); neumann = 1
// adds the Neumann terms (Poisson only) from grad[axis].
int teo_add_bc_to_rhs(const te_level_desc* d, int kind, int neumann, teo_point_fn gfun, teo_point_fn hfun,
                      const teo_point_fn* grad, double* f) {
  return guard([&] {
    Level L(d);
    const int D = L.D;
    for (int p = 0; p < L.P; p++) {
      double* fp = f + p * L.pstride(1);
      for (int side = 0; side < 2 * D; side++) {
        if (L.has(p, D - 1, side)) continue;
        const int axis = side >> 1, upper = side & 1;
        const double h = L.h(p, axis);
        const double h2 = std::pow(h, 2);
        const int t0 = axis == 0 ? 1 : 0, t1 = axis == 2 ? 1 : 2;
        const int m0 = L.n[t0], m1 = D == 3 ? L.n[t1] : 1;
        for (int j = 0; j < m1; j++)
          for (int i = 0; i < m0; i++) {
            double x[3] = {0, 0, 0};
            int c[3] = {0, 0, 0};
            for (int a = 0; a < D; a++) {
              if (a == axis) {
                x[a] = upper ? L.starts[(size_t)p * D + a] + L.spacings[(size_t)p * D + a] * L.n[a]
                             : L.starts[(size_t)p * D + a];
                c[a] = upper ? L.n[a] - 1 : 0;
              } else {
                const int k = a == t0 ? i : j;
                x[a] = L.starts[(size_t)p * D + a] + L.spacings[(size_t)p * D + a] / 2.0 +
                       L.spacings[(size_t)p * D + a] * k;
                c[a] = k;
              }
            }
            double& cell = fp[L.at(c[0], c[1], c[2], 0)];
            if (neumann) {
              if (!upper)
                cell += grad[axis](x) / h;
              else
                cell -= grad[axis](x) / h;
            } else if (kind == 0) {
              cell += -2.0 * gfun(x) / h2;
            } else {
              cell -= 2 * gfun(x) * hfun(x) / h2;
            }
          }
      }
    }
  });
}

// smoother: 0 DFT, 1 BiCGStab patch solver; mode 0 smooth, 1 apply
int teo_patch_solver(const te_level_desc* d, int scheme, int fill_type, int kind, const double* coeffs,
                     int smoother, int dft_neumann_mask, double tol, int max_it, int cont, int mode, int nc,
                     const double* f, double* u, long long* inner_its) {
  return guard([&] {
    Level L(d);
    Op op(L, scheme, fill_type, kind, false, coeffs);
    Smoother* s;
    if (smoother == 0)
      s = new DFTSolver(&op, dft_neumann_mask);
    else
      s = new BiCGStabPatchSolver(&op, tol, max_it, cont != 0);
    try {
      if (mode == 0)
        s->smooth(f, u, nc);
      else
        s->apply(f, u, nc);
    } catch (...) {
      delete s;
      throw;
    }
    if (inner_its && smoother == 1) *inner_its = static_cast<BiCGStabPatchSolver*>(s)->inner_iterations;
    delete s;
  });
}

int teo_restrict(const te_level_desc* fine, const te_level_desc* coarse, int extrapolate, int nc,
                 const double* f, double* c) {
  return guard([&] {
    Level F(fine), C(coarse);
    restrict_vec(F, C, extrapolate != 0, f, c, nc);
  });
}

int teo_interpolate(const te_level_desc* coarse, const te_level_desc* fine, int nc, const double* c,
                    double* f) {
  return guard([&] {
    Level F(fine), C(coarse);
    interpolate_vec(C, F, c, f, nc);
  });
}

static Hierarchy* make_hierarchy(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg,
                                 const double* const* coeffs) {
  auto* H = new Hierarchy();
  H->levels.reserve(nlevels);
  for (int k = 0; k < nlevels; k++) H->levels.emplace_back(&levels[k]);
  for (int k = 0; k < nlevels; k++) {
    Op* op = new Op(H->levels[k], cfg->scheme, cfg->fill_type, cfg->op_kind, cfg->neumann != 0,
                    cfg->op_kind == 1 ? coeffs[k] : nullptr);
    H->ops.push_back(op);
    if (cfg->smoother == 0)
      H->smoothers.push_back(new DFTSolver(op, cfg->dft_neumann_mask));
    else
      H->smoothers.push_back(
          new BiCGStabPatchSolver(op, cfg->inner_tol, cfg->inner_max_it, cfg->inner_continue_on_breakdown != 0));
  }
  H->pre = cfg->pre_sweeps;
  H->post = cfg->post_sweeps;
  H->coarse_sweeps = cfg->coarse_sweeps;
  H->mid = cfg->mid_sweeps;
  if (cfg->cycle_type < 0 || cfg->cycle_type > 2) throw std::runtime_error("unsupported cycle type");
  H->type = cfg->cycle_type;
  H->extrapolate = cfg->extrapolate_boundary_ghosts != 0;
  return H;
}

int teo_vcycle_apply(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg,
                     const double* const* coeffs, int nc, const double* f, double* u) {
  return guard([&] {
    Hierarchy* H = make_hierarchy(levels, nlevels, cfg, coeffs);
    try {
      H->apply(f, u, nc);
    } catch (...) {
      delete H;
      throw;
    }
    delete H;
  });
}

// Iterative::CG::solve (Iterative/CG.h:126-194): right-preconditioned in the
// reference's form -- the iteration runs on a correction started at zero
// (x.set(0) after the initial residual), the preconditioner is applied to the
// search direction before A, and at the end the correction is mapped through
// Mr and the initial guess added back.  A zero right-hand side returns at once
// with x = 0 (the initial guess is not restored there, as in the reference).
int cg(const Space& V, const ApplyFn& A, double* x, const double* b, const ApplyFn* Mr, double tol, int max_it,
       double* final_res, bool* breakdown) {
  *breakdown = false;
  std::vector<double> resid = V.zero();
  A(x, resid.data());
  V.each([&](long i) { resid[i] = resid[i] * -1 + b[i]; });  // scaleThenAdd(-1, b)
  std::vector<double> initial_guess(x, x + V.size());
  V.each([&](long i) { x[i] = 0.0; });  // x.set(0)
  double r0 = V.norm(b);
  std::vector<double> p = resid, ap = V.zero(), tmp;
  if (Mr) tmp = V.zero();
  double rho = V.dot(resid.data(), resid.data());
  int its = 0;
  if (final_res) *final_res = 0.0;
  if (r0 == 0) return its;
  double residual = V.norm(resid.data()) / r0;
  if (final_res) *final_res = residual;
  while (residual > tol && its < max_it) {
    if (rho == 0) {
      *breakdown = true;
      return its;
    }
    if (Mr) {
      std::fill(tmp.begin(), tmp.end(), 0.0);
      (*Mr)(p.data(), tmp.data());
      A(tmp.data(), ap.data());
    } else {
      A(p.data(), ap.data());
    }
    double alpha = rho / V.dot(p.data(), ap.data());
    V.each([&](long i) { x[i] += p[i] * alpha; });           // x.addScaled(alpha, p)
    V.each([&](long i) { resid[i] += ap[i] * -alpha; });     // resid.addScaled(-alpha, ap)
    double rho_new = V.dot(resid.data(), resid.data());
    double beta = rho_new / rho;
    V.each([&](long i) { p[i] = p[i] * beta + resid[i]; });  // p.scaleThenAdd(beta, resid)
    its++;
    rho = rho_new;
    residual = V.norm(resid.data()) / r0;
    if (final_res) *final_res = residual;
  }
  if (Mr) {
    (*Mr)(x, resid.data());
    V.each([&](long i) { x[i] = resid[i]; });  // x.copy(resid)
  }
  V.each([&](long i) { x[i] += initial_guess[i]; });  // x.add(initial_guess)
  return its;
}

// BiCGStab (or CG) with A = finest operator, M = the cycle; returns TE_ERR_BREAKDOWN on rho == 0
int teo_gmg_solve(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg,
                  const double* const* coeffs, int nc, double* u, const double* f, int* iterations,
                  double* final_residual) {
  int status = TE_OK;
  int rc = guard([&] {
    Hierarchy* H = make_hierarchy(levels, nlevels, cfg, coeffs);
    const Level& L = H->levels[0];
    Space V{L, L.P, nc};
    ApplyFn A = [&](double* x, double* b) { H->ops[0]->apply(x, b, nc); };
    ApplyFn M = [&](double* x, double* b) { H->apply(x, b, nc); };
    bool bd = false;
    try {
      if (cfg->krylov == 1)
        *iterations = cg(V, A, u, f, cfg->use_precond ? &M : nullptr, cfg->tol, cfg->max_it, final_residual, &bd);
      else
        *iterations = bicgstab(V, A, u, f, cfg->use_precond ? &M : nullptr, cfg->tol, cfg->max_it,
                               final_residual, &bd, cfg->precond_exit != 0);
    } catch (...) {
      delete H;
      throw;
    }
    if (bd) status = TE_ERR_BREAKDOWN;
    delete H;
  });
  return rc != TE_OK ? rc : status;
}

}  // extern "C"
