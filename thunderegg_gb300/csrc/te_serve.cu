// te_serve.cu -- continuous batching of independent Poisson solves behind the
// C ABI (te_serve_*; no counterpart in the reference, whose solvers run one
// solve per Iterative::BiCGStab::solve call).  The scheduler is host code over
// the library's own entry points: per-request mesh tables are copied at
// submit, requests that share patch shape and solver options form a class,
// and a class's active requests are packed into one union hierarchy (the
// members' level tables concatenated with shifted ids, shallower members
// padded with copies of their coarsest level) whose resumable slot-mode
// BiCGStab batch (te_bicgstab_batch_*) every round advances a few iterations.
// Between steps a round admits queued requests against the memory budget,
// starts waiting requests in free slots built on their mesh, finishes the
// solves that stopped and re-forms a class's batch when requests wait without
// a slot of their mesh (continuing solves restart from their current
// iterates).  Unions are cached by their members' meshes, so their captured
// CUDA graphs are replayed, and idle ones are evicted least recently used.
//
// One thread drives a server (its calls are not thread safe); its handles
// bind to the stream that was current (te_set_stream) when it was created.

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "te_internal.cuh"

namespace {

using te::Error;
using te::require;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int face_slots(int dim) { return dim == 2 ? 8 : 26; }

// one level of a mesh, owned (te_level_desc points into it)
struct MeshLevel {
  int dim = 2, ns[3] = {1, 1, 1}, g = 1, P = 0;
  std::vector<int> id, refine, parent, orth, child, nbr_type, nbr_ids, nbr_orth;
  std::vector<double> starts, spacings;

  int nchild() const { return 1 << dim; }
  long long padded_cells() const {
    long long c = 1;
    for (int a = 0; a < dim; a++) c *= ns[a] + 2 * g;
    return c;
  }
  te_level_desc desc() const {
    te_level_desc d;
    d.dim = dim;
    for (int a = 0; a < 3; a++) d.ns[a] = ns[a];
    d.num_ghost = g;
    d.num_patches = P;
    d.id = id.data();
    d.refine_level = refine.data();
    d.parent_id = parent.data();
    d.orth_on_parent = orth.data();
    d.child_ids = child.data();
    d.starts = starts.data();
    d.spacings = spacings.data();
    d.nbr_type = nbr_type.data();
    d.nbr_ids = nbr_ids.data();
    d.nbr_orth = nbr_orth.data();
    return d;
  }
};
using Mesh = std::vector<MeshLevel>;

template <class T>
std::vector<T> copy_arr(const T* p, size_t n, const char* what) {
  require(p != nullptr || n == 0, std::string("te_serve_submit: null ") + what);
  return std::vector<T>(p, p + n);
}

MeshLevel copy_level(const te_level_desc& d) {
  require(d.dim == 2 || d.dim == 3, "te_serve_submit: dim must be 2 or 3");
  require(d.num_patches > 0 && d.num_ghost >= 1, "te_serve_submit: empty level or no ghost layer");
  MeshLevel L;
  L.dim = d.dim;
  for (int a = 0; a < 3; a++) L.ns[a] = a < d.dim ? d.ns[a] : 1;
  for (int a = 0; a < d.dim; a++) require(L.ns[a] > 0, "te_serve_submit: bad patch size");
  L.g = d.num_ghost;
  L.P = d.num_patches;
  const size_t P = (size_t)L.P, F = (size_t)face_slots(d.dim);
  L.id = copy_arr(d.id, P, "id");
  L.refine = copy_arr(d.refine_level, P, "refine_level");
  L.parent = copy_arr(d.parent_id, P, "parent_id");
  L.orth = copy_arr(d.orth_on_parent, P, "orth_on_parent");
  L.child = copy_arr(d.child_ids, P << d.dim, "child_ids");
  L.starts = copy_arr(d.starts, P * d.dim, "starts");
  L.spacings = copy_arr(d.spacings, P * d.dim, "spacings");
  L.nbr_type = copy_arr(d.nbr_type, P * F, "nbr_type");
  L.nbr_ids = copy_arr(d.nbr_ids, P * F * 4, "nbr_ids");
  L.nbr_orth = copy_arr(d.nbr_orth, P * F, "nbr_orth");
  return L;
}

// FNV-1a over the tables: requests on equal meshes share unions and slots
struct Hasher {
  uint64_t h = 1469598103934665603ull;
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) {
      h ^= c[i];
      h *= 1099511628211ull;
    }
  }
  template <class T>
  void vec(const std::vector<T>& v) {
    const uint64_t n = v.size();
    bytes(&n, sizeof n);
    bytes(v.data(), v.size() * sizeof(T));
  }
};

uint64_t mesh_key(const Mesh& m) {
  Hasher H;
  for (const MeshLevel& L : m) {
    const int hdr[6] = {L.dim, L.ns[0], L.ns[1], L.ns[2], L.g, L.P};
    H.bytes(hdr, sizeof hdr);
    H.vec(L.id);
    H.vec(L.refine);
    H.vec(L.parent);
    H.vec(L.orth);
    H.vec(L.child);
    H.vec(L.starts);
    H.vec(L.spacings);
    H.vec(L.nbr_type);
    H.vec(L.nbr_ids);
    H.vec(L.nbr_orth);
  }
  return H.h;
}

// The hierarchy extended to `depth` levels by repeating its coarsest level: each new level's
// patch is the old coarsest patch (its own parent, no orthant, one child), the reference's rule
// for patches that are not coarsened (P4estDomainGenerator.cpp:272-321)
Mesh pad_mesh(const Mesh& m, int depth) {
  Mesh out = m;
  while ((int)out.size() < depth) {
    const MeshLevel c = out.back();
    MeshLevel fine = c, coarse = c;
    fine.parent = c.id;
    std::fill(fine.orth.begin(), fine.orth.end(), -1);
    std::fill(coarse.parent.begin(), coarse.parent.end(), -1);
    std::fill(coarse.orth.begin(), coarse.orth.end(), -1);
    std::fill(coarse.child.begin(), coarse.child.end(), -1);
    for (int p = 0; p < c.P; p++) coarse.child[(size_t)p * c.nchild()] = c.id[p];
    out.back() = fine;
    out.push_back(coarse);
  }
  return out;
}

// the members' levels concatenated, every id shifted past the previous members' ids
Mesh union_mesh(const std::vector<const Mesh*>& ms, std::vector<std::vector<int>>& offsets) {
  size_t depth = 0;
  for (const Mesh* m : ms) depth = std::max(depth, m->size());
  std::vector<Mesh> padded;
  for (const Mesh* m : ms) padded.push_back(pad_mesh(*m, (int)depth));
  std::vector<long long> shift;
  long long acc = 0;
  for (const Mesh& m : padded) {
    shift.push_back(acc);
    int mx = -1;
    for (const MeshLevel& L : m)
      for (int v : L.id) mx = std::max(mx, v);
    acc += (long long)mx + 1;
  }
  require(acc <= 0x7fffffffll, "te_serve: the union's patch ids exceed the int range");
  Mesh out(depth);
  offsets.assign(depth, {});
  for (size_t k = 0; k < depth; k++) {
    MeshLevel& U = out[k];
    const MeshLevel& L0 = padded[0][k];
    U.dim = L0.dim;
    for (int a = 0; a < 3; a++) U.ns[a] = L0.ns[a];
    U.g = L0.g;
    U.P = 0;
    offsets[k].push_back(0);
    const int F = face_slots(U.dim);
    for (size_t b = 0; b < padded.size(); b++) {
      const MeshLevel& L = padded[b][k];
      const int s = (int)shift[b];
      auto sh = [s](int v) { return v >= 0 ? v + s : v; };
      for (int p = 0; p < L.P; p++) {
        U.id.push_back(L.id[p] + s);
        U.refine.push_back(L.refine[p]);
        U.parent.push_back(sh(L.parent[p]));
        U.orth.push_back(L.orth[p]);
        for (int c = 0; c < L.nchild(); c++) U.child.push_back(sh(L.child[(size_t)p * L.nchild() + c]));
        for (int a = 0; a < L.dim; a++) {
          U.starts.push_back(L.starts[(size_t)p * L.dim + a]);
          U.spacings.push_back(L.spacings[(size_t)p * L.dim + a]);
        }
        for (int f = 0; f < F; f++) {
          const size_t q = (size_t)p * F + f;
          const int t = L.nbr_type[q];
          U.nbr_type.push_back(t);
          U.nbr_orth.push_back(L.nbr_orth[q]);
          for (int j = 0; j < 4; j++) {
            const int v = L.nbr_ids[q * 4 + j];
            U.nbr_ids.push_back(t >= 0 && v >= 0 ? v + s : v);
          }
        }
      }
      U.P += L.P;
      offsets[k].push_back(U.P);
    }
  }
  return out;
}

// device memory a request holds while active: the cycle's work buffers on every level, the
// finest level's Krylov vectors, iterate and right-hand side, and the level tables
double request_bytes(const Mesh& m, const te_solve_opts& o) {
  const double w = o.cycle_dtype == TE_F64 ? 8 : 4;
  double total = 0;
  for (size_t k = 0; k < m.size(); k++) {
    const MeshLevel& L = m[k];
    const double cells = (double)L.P * L.padded_cells();
    double face = 1;
    for (int a = 1; a < L.dim; a++) face *= L.ns[0];
    total += cells * 3 * w + (double)L.P * 2 * L.dim * face * 4 + (double)L.P * 512;
    if (k == 0) total += cells * (8 * 8 + 8 * 3 + 8);
  }
  return total;
}

int bucket(int n) {
  static const int b[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256};
  for (int v : b)
    if (v >= n) return v;
  return n;
}

struct Req {
  long long id = 0;
  std::shared_ptr<const Mesh> mesh;
  uint64_t key = 0;
  te_solve_opts o{};
  std::string ckey;
  std::vector<double> f;  // finest level, padded layout
  std::vector<double> x;  // current iterate between batches (empty: zero)
  double t_submit = 0, bytes = 0;
  int iterations = 0, restarts = 0;
};

struct Done {
  std::vector<double> u;
  te_serve_result r{};
};

// the device objects of one union hierarchy and its batch buffers
struct Union {
  std::string key;
  std::vector<uint64_t> members;
  std::vector<te_domain*> dom;
  std::vector<te_ghost_filler*> gf;
  std::vector<te_operator*> op;
  std::vector<te_patch_solver*> sm;
  std::vector<te_restrictor*> rs;
  std::vector<te_interpolator*> ip;
  te_cycle* cycle = nullptr;
  void* x = nullptr;
  void* b = nullptr;
  std::vector<int> offs;  // finest patch offsets of the slots
  long long pstride = 0;  // doubles per finest patch
  double bytes = 0;
  ~Union() {
    if (cycle) te_cycle_destroy(cycle);
    for (auto* p : ip)
      if (p) te_interpolator_destroy(p);
    for (auto* p : rs)
      if (p) te_restrictor_destroy(p);
    for (auto* p : sm)
      if (p) te_patch_solver_destroy(p);
    for (auto* p : op)
      if (p) te_operator_destroy(p);
    for (auto* p : gf)
      if (p) te_ghost_filler_destroy(p);
    if (x) te_level_free(x);
    if (b) te_level_free(b);
    for (auto* p : dom)
      if (p) te_domain_destroy(p);
  }
};

void chk(int rc, const char* what) {
  if (rc != TE_OK) throw Error(rc, std::string(what) + ": " + te_last_error_message());
}

std::unique_ptr<Union> build_union(const std::vector<const Mesh*>& ms, const te_solve_opts& o) {
  std::vector<std::vector<int>> offsets;
  const Mesh U = union_mesh(ms, offsets);
  auto un = std::make_unique<Union>();
  const int n = (int)U.size();
  for (int k = 0; k < n; k++) {
    const te_level_desc d = U[k].desc();
    te_domain* dm = nullptr;
    chk(te_domain_create(&d, &dm), "te_serve: domain");
    un->dom.push_back(dm);
    te_ghost_filler* g = nullptr;
    chk(te_ghost_filler_create(dm, o.scheme, o.fill_type, &g), "te_serve: ghost filler");
    un->gf.push_back(g);
    te_operator* op = nullptr;
    chk(te_poisson_operator_create(dm, g, 0, &op), "te_serve: operator");
    un->op.push_back(op);
    te_patch_solver* s = nullptr;
    if (o.smoother == 0) {
      const MeshLevel& L = U[k];
      const bool cube = L.g == 1 && L.ns[1] == L.ns[0] && (L.dim == 2 || L.ns[2] == L.ns[0]);
      const bool tc = cube && ((L.dim == 2 && (L.ns[0] == 16 || L.ns[0] == 32 || L.ns[0] == 64)) ||
                               (L.dim == 3 && L.ns[0] == 16));
      if (o.tc_precision == TE_TC_BF16 && tc)
        chk(te_dft_patch_solver_create_tc(op, 0, TE_TC_BF16, &s), "te_serve: patch solver");
      else
        chk(te_dft_patch_solver_create(op, 0, &s), "te_serve: patch solver");
    } else {
      chk(te_bicgstab_patch_solver_create(op, o.inner_tol, o.inner_max_iterations, o.inner_continue_on_breakdown,
                                          &s),
          "te_serve: patch solver");
    }
    un->sm.push_back(s);
  }
  un->ip.push_back(nullptr);
  for (int k = 0; k + 1 < n; k++) {
    te_restrictor* r = nullptr;
    chk(te_linear_restrictor_create(un->dom[k], un->dom[k + 1], 0, &r), "te_serve: restrictor");
    un->rs.push_back(r);
    te_interpolator* i = nullptr;
    chk(te_direct_interpolator_create(un->dom[k + 1], un->dom[k], &i), "te_serve: interpolator");
    un->ip.push_back(i);
  }
  un->rs.push_back(nullptr);
  std::vector<te_cycle_level> lv(n);
  for (int k = 0; k < n; k++) lv[k] = {un->op[k], un->sm[k], un->rs[k], un->ip[k]};
  te_cycle_opts co{o.pre_sweeps, o.post_sweeps, 1, o.coarse_sweeps};
  chk(te_cycle_create(lv.data(), n, co, TE_CYCLE_V, o.cycle_dtype, &un->cycle), "te_serve: cycle");
  chk(te_level_alloc(un->dom[0], 1, TE_F64, &un->x), "te_serve: x");
  chk(te_level_alloc(un->dom[0], 1, TE_F64, &un->b), "te_serve: b");
  un->offs = offsets[0];
  un->pstride = te_domain_patch_stride(un->dom[0], 1);
  for (const Mesh* m : ms) un->bytes += request_bytes(*m, o);
  return un;
}

struct Class {
  std::deque<Req*> waiting;
  std::unique_ptr<Union> un;
  te_bicgstab_batch* batch = nullptr;
  std::vector<Req*> slot;             // request in each slot (null: free)
  std::vector<std::shared_ptr<const Mesh>> slot_mesh;
  std::vector<uint64_t> slot_key;
  int wait_rounds = 0;
};

std::string class_key(const Mesh& m, const te_solve_opts& o) {
  const MeshLevel& L = m[0];
  char buf[512];
  std::snprintf(buf, sizeof buf, "%d|%d,%d,%d|%d|%d,%d,%d,%.17g,%d,%d,%d,%d,%d,%.17g,%d,%d,%d,%d", L.dim, L.ns[0],
                L.ns[1], L.ns[2], L.g, o.scheme, o.fill_type, o.smoother, o.inner_tol, o.inner_max_iterations,
                o.inner_continue_on_breakdown, o.pre_sweeps, o.post_sweeps, o.coarse_sweeps, o.tol, o.max_iterations,
                o.cycle_dtype, o.flags, o.tc_precision);
  return buf;
}

}  // namespace

struct te_server {
  te_serve_opts o{};
  cudaStream_t st = nullptr;
  long long next_id = 1;
  std::deque<std::unique_ptr<Req>> queue;           // submitted, not admitted
  std::map<long long, std::unique_ptr<Req>> live;   // admitted, not finished
  std::map<std::string, Class> classes;
  std::list<std::unique_ptr<Union>> idle;           // cached unions, most recently used first
  std::map<long long, Done> done;
  double live_bytes = 0;                            // estimate of the admitted requests
  te_serve_counters c{};

  double idle_bytes() const {
    double s = 0;
    for (const auto& u : idle) s += u->bytes;
    return s;
  }

  ~te_server() {
    for (auto& kv : classes)
      if (kv.second.batch) te_bicgstab_batch_destroy(kv.second.batch);
  }

  std::unique_ptr<Union> take_union(const std::string& key, const std::vector<uint64_t>& members,
                                    const std::vector<const Mesh*>& ms, const te_solve_opts& so) {
    for (auto it = idle.begin(); it != idle.end(); ++it)
      if ((*it)->key == key && (*it)->members == members) {
        std::unique_ptr<Union> u = std::move(*it);
        idle.erase(it);
        c.union_cache_hits++;
        return u;
      }
    // the new union holds admitted requests (counted in live_bytes) and free slots the budget
    // had room for: idle unions give way, least recently used first
    while (!idle.empty() && live_bytes + idle_bytes() > o.budget_bytes) idle.pop_back();
    c.union_builds++;
    const double t0 = now_s();
    auto u = build_union(ms, so);
    c.build_s += now_s() - t0;
    u->key = key;
    u->members = members;
    return u;
  }
  void park(std::unique_ptr<Union> u) {
    if (!u) return;
    idle.push_front(std::move(u));
    while (!idle.empty() && live_bytes + idle_bytes() > o.budget_bytes) idle.pop_back();
  }

  void put_slot(Union& u, int slot, const Req* r) {
    const size_t off = (size_t)u.offs[slot] * u.pstride, len = (size_t)(u.offs[slot + 1] - u.offs[slot]) * u.pstride;
    double* xb = static_cast<double*>(u.x) + off;
    double* bb = static_cast<double*>(u.b) + off;
    if (r) {
      require(r->f.size() == len, "te_serve: right-hand side size");
      TE_CUDA(cudaMemcpyAsync(bb, r->f.data(), len * sizeof(double), cudaMemcpyHostToDevice, st));
      if (r->x.size() == len)
        TE_CUDA(cudaMemcpyAsync(xb, r->x.data(), len * sizeof(double), cudaMemcpyHostToDevice, st));
      else
        TE_CUDA(cudaMemsetAsync(xb, 0, len * sizeof(double), st));
    } else {
      TE_CUDA(cudaMemsetAsync(bb, 0, len * sizeof(double), st));
      TE_CUDA(cudaMemsetAsync(xb, 0, len * sizeof(double), st));
    }
  }

  void get_slot(const Union& u, int slot, std::vector<double>& out) {
    const size_t off = (size_t)u.offs[slot] * u.pstride, len = (size_t)(u.offs[slot + 1] - u.offs[slot]) * u.pstride;
    out.resize(len);
    TE_CUDA(cudaMemcpyAsync(out.data(), static_cast<const double*>(u.x) + off, len * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
    TE_CUDA(cudaStreamSynchronize(st));
  }

  // a new batch for the class: its running requests (iterates carried over) and waiting ones
  void reform(const std::string& ck, Class& cl) {
    const double t0 = now_s(), b0 = c.build_s;
    reform_(ck, cl);
    c.form_s += (now_s() - t0) - (c.build_s - b0);
  }
  void reform_(const std::string& ck, Class& cl) {
    std::vector<Req*> members;
    if (cl.batch) {
      chk(te_bicgstab_batch_sync_x(cl.batch), "te_serve: sync");
      std::vector<int> its(cl.slot.size());
      chk(te_bicgstab_batch_state(cl.batch, its.data(), nullptr, nullptr, nullptr), "te_serve: state");
      for (size_t s = 0; s < cl.slot.size(); s++)
        if (Req* r = cl.slot[s]) {
          get_slot(*cl.un, (int)s, r->x);
          r->iterations += its[s];
          r->restarts++;
          members.push_back(r);
        }
      chk(te_bicgstab_batch_destroy(cl.batch), "te_serve: batch");
      cl.batch = nullptr;
      park(std::move(cl.un));
    }
    while (!cl.waiting.empty() && (int)members.size() < o.max_batch) {
      members.push_back(cl.waiting.front());
      cl.waiting.pop_front();
    }
    // slots in mesh order: a class that meets the same set of meshes again gets the same union
    // key, so its cached union (and the union's captured graphs) are reused
    std::stable_sort(members.begin(), members.end(), [](const Req* a, const Req* b) { return a->key < b->key; });
    cl.slot.clear();
    cl.slot_mesh.clear();
    cl.slot_key.clear();
    if (members.empty()) return;
    // round up to a bucket size with free slots on the last member's mesh, when the budget allows
    int nslots = (int)members.size();
    const int want = std::min(bucket(nslots), std::max(nslots, o.max_batch));
    const double per = members.back()->bytes;
    while (nslots < want && live_bytes + idle_bytes() + per * (nslots + 1 - (int)members.size()) <= o.budget_bytes)
      nslots++;
    std::vector<const Mesh*> ms;
    std::vector<uint64_t> keys;
    for (int s = 0; s < nslots; s++) {
      const Req* r = members[std::min(s, (int)members.size() - 1)];
      ms.push_back(r->mesh.get());
      keys.push_back(r->key);
      cl.slot.push_back(s < (int)members.size() ? members[s] : nullptr);
      cl.slot_mesh.push_back(r->mesh);
      cl.slot_key.push_back(r->key);
    }
    cl.un = take_union(ck, keys, ms, members[0]->o);
    for (int s = 0; s < nslots; s++) put_slot(*cl.un, s, cl.slot[s]);
    const te_solve_opts& so = members[0]->o;
    chk(te_bicgstab_batch_create(cl.un->op[0], 1, cl.un->x, cl.un->b, cl.un->cycle, so.tol, so.max_iterations,
                                 so.flags | TE_BICGSTAB_SLOTS, nslots, cl.un->offs.data(), &cl.batch),
        "te_serve: batch");
    cl.wait_rounds = 0;
    c.reforms++;
  }

  void finish(Class& cl, int s, int its, double res, int status) {
    Req* r = cl.slot[s];
    Done d;
    get_slot(*cl.un, s, d.u);
    d.r.status = status;
    d.r.iterations = r->iterations + its;
    d.r.residual = res;
    d.r.latency_s = now_s() - r->t_submit;
    d.r.restarts = r->restarts;
    done[r->id] = std::move(d);
    live_bytes -= r->bytes;
    c.completed++;
    cl.slot[s] = nullptr;
    live.erase(r->id);
  }

  int round() {
    c.rounds++;
    // 1. admission against the budget (idle unions give way)
    while (!queue.empty()) {
      Req* r = queue.front().get();
      while (!idle.empty() && live_bytes + idle_bytes() + r->bytes > o.budget_bytes) idle.pop_back();
      if (live_bytes + r->bytes > o.budget_bytes && live_bytes > 0) break;
      std::unique_ptr<Req> up = std::move(queue.front());
      queue.pop_front();
      live_bytes += r->bytes;
      classes[r->ckey].waiting.push_back(r);
      live[r->id] = std::move(up);
      c.admitted++;
    }
    for (auto& kv : classes) {
      Class& cl = kv.second;
      // 2. waiting requests into free slots built on their mesh
      if (cl.batch) {
        std::vector<int> running(cl.slot.size());
        chk(te_bicgstab_batch_state(cl.batch, nullptr, nullptr, nullptr, running.data()), "te_serve: state");
        for (size_t s = 0; s < cl.slot.size() && !cl.waiting.empty(); s++) {
          if (cl.slot[s] || running[s]) continue;
          for (auto it = cl.waiting.begin(); it != cl.waiting.end(); ++it)
            if ((*it)->key == cl.slot_key[s]) {
              cl.slot[s] = *it;
              cl.waiting.erase(it);
              put_slot(*cl.un, (int)s, cl.slot[s]);
              chk(te_bicgstab_batch_reset(cl.batch, (int)s), "te_serve: reset");
              c.slot_fills++;
              break;
            }
        }
      }
      // 3. a new batch when requests wait without a slot of their mesh
      if (!cl.waiting.empty()) {
        int occupied = 0;
        for (Req* r : cl.slot) occupied += r != nullptr;
        if (!cl.batch || occupied == 0 || 2 * (int)cl.waiting.size() >= (int)cl.slot.size() || cl.wait_rounds >= 2)
          reform(kv.first, cl);
        else
          cl.wait_rounds++;
      }
      // 4. iterate, then finish the solves that stopped
      if (!cl.batch) continue;
      int nrun = 0;
      const double t0 = now_s();
      chk(te_bicgstab_batch_step(cl.batch, std::max(1, o.steps_per_round), &nrun), "te_serve: step");
      const double t1 = now_s();
      c.step_s += t1 - t0;
      const size_t B = cl.slot.size();
      std::vector<int> its(B), sts(B), running(B);
      std::vector<double> res(B);
      chk(te_bicgstab_batch_state(cl.batch, its.data(), res.data(), sts.data(), running.data()), "te_serve: state");
      std::vector<int> stop;
      for (size_t s = 0; s < B; s++)
        if (cl.slot[s] && !running[s]) stop.push_back((int)s);
      if (!stop.empty()) {
        std::vector<int> fin(stop.size());
        chk(te_bicgstab_batch_finish_slots(cl.batch, (int)stop.size(), stop.data(), fin.data()), "te_serve: finish");
        chk(te_bicgstab_batch_state(cl.batch, its.data(), res.data(), sts.data(), running.data()), "te_serve: state");
        for (size_t k = 0; k < stop.size(); k++)
          if (fin[k]) finish(cl, stop[k], its[stop[k]], res[stop[k]], sts[stop[k]]);
      }
      c.finish_s += now_s() - t1;
      // an empty batch goes back to the cache
      bool any = false;
      for (Req* r : cl.slot) any = any || r;
      if (!any && cl.waiting.empty()) {
        chk(te_bicgstab_batch_destroy(cl.batch), "te_serve: batch");
        cl.batch = nullptr;
        cl.slot.clear();
        cl.slot_mesh.clear();
        cl.slot_key.clear();
        park(std::move(cl.un));
      }
    }
    return (int)(queue.size() + live.size());
  }
};

using namespace te;

extern "C" {

int te_serve_create(const te_serve_opts* opts, te_server** out) {
  return guard([&] {
    require(opts && out, "te_serve_create: null argument");
    require(opts->budget_bytes > 0, "te_serve_create: budget_bytes must be positive");
    require(opts->max_batch >= 1, "te_serve_create: max_batch must be >= 1");
    auto s = std::make_unique<te_server>();
    s->o = *opts;
    if (s->o.steps_per_round < 1) s->o.steps_per_round = 1;
    s->st = current_stream();
    *out = s.release();
  });
}

int te_serve_destroy(te_server* s) {
  return guard([&] {
    if (!s) return;
    cudaStream_t prev = current_stream();
    te_set_stream(s->st);
    delete s;
    te_set_stream(prev);
  });
}

int te_serve_submit(te_server* s, const te_level_desc* levels, int num_levels, const te_solve_opts* opts,
                    const double* f, long long* request_id) {
  return guard([&] {
    require(s && levels && opts && f && request_id, "te_serve_submit: null argument");
    require(num_levels >= 1, "te_serve_submit: no levels");
    auto m = std::make_shared<Mesh>();
    for (int k = 0; k < num_levels; k++) m->push_back(copy_level(levels[k]));
    for (int k = 1; k < num_levels; k++)
      require((*m)[k].dim == (*m)[0].dim && (*m)[k].ns[0] == (*m)[0].ns[0] && (*m)[k].ns[1] == (*m)[0].ns[1] &&
                  (*m)[k].ns[2] == (*m)[0].ns[2] && (*m)[k].g == (*m)[0].g,
              "te_serve_submit: levels of one request must share patch shape");
    require(opts->cycle_dtype == TE_F64 || opts->cycle_dtype == TE_F32, "te_serve_submit: bad cycle_dtype");
    require(opts->tol > 0 && opts->max_iterations >= 0, "te_serve_submit: bad tolerance or iteration limit");
    auto r = std::make_unique<Req>();
    r->o = *opts;
    r->bytes = request_bytes(*m, *opts);
    if (r->bytes > s->o.budget_bytes) {
      s->c.rejected++;
      throw Error(TE_ERR_BUDGET, "te_serve_submit: the request needs more device memory than the whole budget");
    }
    const MeshLevel& L0 = (*m)[0];
    r->f.assign(f, f + (size_t)L0.P * L0.padded_cells());
    r->key = mesh_key(*m);
    r->ckey = class_key(*m, *opts);
    r->mesh = m;
    r->id = s->next_id++;
    r->t_submit = now_s();
    *request_id = r->id;
    s->queue.push_back(std::move(r));
    s->c.submitted++;
  });
}

int te_serve_step(te_server* s, int* unfinished) {
  return guard([&] {
    require(s != nullptr, "te_serve_step: null server");
    cudaStream_t prev = current_stream();
    te_set_stream(s->st);
    try {
      const int n = s->round();
      if (unfinished) *unfinished = n;
    } catch (...) {
      te_set_stream(prev);
      throw;
    }
    te_set_stream(prev);
  });
}

int te_serve_poll(te_server* s, long long request_id, double* u, te_serve_result* result) {
  int pending = 0;
  const int rc = guard([&] {
    require(s != nullptr, "te_serve_poll: null server");
    auto it = s->done.find(request_id);
    if (it == s->done.end()) {
      bool known = s->live.count(request_id) > 0;
      for (const auto& q : s->queue) known = known || q->id == request_id;
      require(known, "te_serve_poll: unknown request id (never submitted, or already returned)");
      pending = 1;
      return;
    }
    if (u) std::memcpy(u, it->second.u.data(), it->second.u.size() * sizeof(double));
    if (result) *result = it->second.r;
    s->done.erase(it);
  });
  return rc == TE_OK && pending ? TE_PENDING : rc;
}

int te_serve_stats(const te_server* s, te_serve_counters* out) {
  return guard([&] {
    require(s && out, "te_serve_stats: null argument");
    *out = s->c;
    out->queued = (int)s->queue.size();
    out->active = (int)s->live.size();
    out->classes = (int)s->classes.size();
    out->bytes_in_use = s->live_bytes + s->idle_bytes();
  });
}

}  // extern "C"
