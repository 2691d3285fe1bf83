// te_krylov.cu -- the outer Iterative::BiCGStab (Iterative/BiCGStab.h:111-203) in FP64.
//
// The reference keeps alpha, omega, rho and beta on the host and reduces with
// MPI_Allreduce after every dot product.  Here all scalars live in device
// memory: each vector update is fused with the dot products that follow it,
// the last block of each reduction finalises the scalars in a fixed order,
// and the host reads the scalars back once per iteration to test for
// convergence or breakdown.  One iteration (two preconditioner applications,
// two operator applications, five fused kernels) is captured into a CUDA
// graph per (x, b, M) and replayed.
//
// Arithmetic per element follows the reference's operation order:
//   s = r + ap*(-alpha); x += mp*alpha + ms*omega; r += ap*(-alpha) + as*(-omega);
//   p += ap*(-omega); p = p*beta + r.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "te_gmg.cuh"

namespace te {

enum Slot {
  S_RHO = 0,
  S_R0,
  S_RHAT_AP,
  S_ALPHA,
  S_SS,
  S_AS_S,
  S_AS_AS,
  S_OMEGA,
  S_RR,
  S_R_RHAT,
  S_BETA,
  S_DONE,
  S_BB,
  S_NSLOTS = 16
};

constexpr int KT = 256;

__device__ __forceinline__ int k_interior_offset(const Layout& L, int e) {
  int x = e % L.n0;
  int r = e / L.n0;
  int y = r % L.n1;
  int z = r / L.n1;
  return L.at(x, y, z);
}

template <int NV>
__device__ void k_reduce(double (&v)[NV], double* part, unsigned int* counter, double* S, int slot0,
                         int finalize_kind, double tol) {
  // finalize_kind: 1 alpha, 2 omega, 3 beta + rho commit, 4 initial r0, 5 early-exit test
  __shared__ double red[NV][KT / 32];
  __shared__ double fin[NV][KT];
  __shared__ bool last;
#pragma unroll
  for (int i = 0; i < NV; i++) {
    double x = v[i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[i][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < NV; i++) {
      double s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[i][w];
      part[(size_t)i * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    unsigned int done = atomicAdd(counter, 1u);
    last = done == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // fixed-order final sum over the block partials: strided per-thread sums,
  // then a fixed tree (blockDim.x is a power of two)
  for (int i = 0; i < NV; i++) {
    double s = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(&part[(size_t)i * gridDim.x + b]);
    fin[i][threadIdx.x] = s;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int i = 0; i < NV; i++) fin[i][threadIdx.x] += fin[i][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double tot[NV];
    for (int i = 0; i < NV; i++) {
      tot[i] = fin[i][0];
      S[slot0 + i] = tot[i];
    }
    if (finalize_kind == 1) {  // alpha = rho / (rhat . ap)
      S[S_ALPHA] = S[S_RHO] / tot[0];
    } else if (finalize_kind == 2) {  // omega = (as . s) / (as . as)
      S[S_OMEGA] = tot[0] / tot[1];
    } else if (finalize_kind == 3) {  // beta = rho_new * alpha / (rho * omega); rho = rho_new
      if (S[S_DONE] == 0.0) {
        S[S_BETA] = S[S_R_RHAT] * S[S_ALPHA] / (S[S_RHO] * S[S_OMEGA]);
        S[S_RHO] = S[S_R_RHAT];
      }
    } else if (finalize_kind == 4) {  // initial: r0 = ||b||
      S[S_R0] = sqrt(S[S_BB]);
    } else if (finalize_kind == 5) {  // ||s|| / ||b|| <= tol (BiCGStab.h:162)
      S[S_DONE] = sqrt(tot[0]) / S[S_R0] <= tol ? 1.0 : 0.0;
    }
    *counter = 0u;
  }
}

// dots of up to three pairs into S[slot0 ...]
template <int NV>
__global__ void __launch_bounds__(KT) k_dots(Layout L, int npc, const double* a0, const double* b0, const double* a1,
                                             const double* b1, const double* a2, const double* b2, double* part,
                                             unsigned int* counter, double* S, int slot0, int fin) {
  double v[NV];
  for (int i = 0; i < NV; i++) v[i] = 0;
  const int N = L.interior();
  for (int pc = blockIdx.x; pc < npc; pc += gridDim.x) {
    long long base = (long long)pc * L.cs;
#pragma unroll 4
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      long long k = base + k_interior_offset(L, e);
      v[0] += a0[k] * b0[k];
      if (NV > 1) v[1] += a1[k] * b1[k];
      if (NV > 2) v[2] += a2[k] * b2[k];
    }
  }
  k_reduce<NV>(v, part, counter, S, slot0, fin, 0);
}

// s = r + ap * (-alpha);  S_SS = s . s; S_DONE = (||s|| / ||b|| <= tol)
__global__ void __launch_bounds__(KT) k_s(Layout L, int npc, double tol, const double* r, const double* ap,
                                          double* s, double* part, unsigned int* counter, double* S) {
  const double alpha = S[S_ALPHA];
  double v[1] = {0};
  const int N = L.interior();
  for (int pc = blockIdx.x; pc < npc; pc += gridDim.x) {
    long long base = (long long)pc * L.cs;
#pragma unroll 4
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      long long k = base + k_interior_offset(L, e);
      double sv = r[k];
      sv += ap[k] * -alpha;
      s[k] = sv;
      v[0] += sv * sv;
    }
  }
  k_reduce<1>(v, part, counter, S, S_SS, 5, tol);
}

// early exit when ||s|| / ||b|| <= tol: x += dir * alpha (reference: dir = p);
// otherwise x += mp*alpha + ms*omega, r += ap*(-alpha) + as*(-omega) and
// the dots r.rhat, r.r; the last block forms beta and commits rho.
__global__ void __launch_bounds__(KT) k_xr(Layout L, int npc, double* x, double* r, const double* mp,
                                           const double* ms, const double* ap, const double* as, const double* rhat,
                                           const double* dir, double* part, unsigned int* counter, double* S) {
  const double alpha = S[S_ALPHA], omega = S[S_OMEGA];
  const bool done = S[S_DONE] != 0.0;
  double v[2] = {0, 0};
  const int N = L.interior();
  for (int pc = blockIdx.x; pc < npc; pc += gridDim.x) {
    long long base = (long long)pc * L.cs;
#pragma unroll 4
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      long long k = base + k_interior_offset(L, e);
      if (done) {
        x[k] += dir[k] * alpha;
      } else {
        x[k] += mp[k] * alpha + ms[k] * omega;
        double rv = r[k];
        rv += ap[k] * -alpha + as[k] * -omega;
        r[k] = rv;
        v[0] += rv * rv;
        v[1] += rv * rhat[k];
      }
    }
  }
  k_reduce<2>(v, part, counter, S, S_RR, 3, 0);
}

// p += ap*(-omega); p = p*beta + r
__global__ void __launch_bounds__(KT) k_p(Layout L, int npc, double* p, const double* ap, const double* r,
                                          const double* S) {
  if (S[S_DONE] != 0.0) return;
  const double omega = S[S_OMEGA], beta = S[S_BETA];
  const int N = L.interior();
  for (int pc = blockIdx.x; pc < npc; pc += gridDim.x) {
    long long base = (long long)pc * L.cs;
#pragma unroll 4
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      long long k = base + k_interior_offset(L, e);
      double pv = p[k];
      pv += ap[k] * -omega;
      p[k] = pv * beta + r[k];
    }
  }
}

struct KrylovWork {
  const te_domain* d;
  int nc;
  size_t n;
  DevBuf<double> resid, rhat, p, ap, as, s, ms, mp, S, part;
  DevBuf<unsigned int> counter;
  double* h = nullptr;
  cudaStream_t cap = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  int grid = 1;
  struct G {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    long long launches = 0;
  };
  // keyed by x, b, the cycle's serial number and buffer generation, tol, flags
  std::map<std::tuple<void*, const void*, unsigned long long, unsigned long long, double, int>, G> graphs;
  KrylovWork(const te_domain* d, int nc) : d(d), nc(nc) {
    n = (size_t)d->lay.P * d->lay.pstride(nc);
    for (auto* b : {&resid, &rhat, &p, &ap, &as, &s, &ms, &mp}) {
      b->alloc(n);
      TE_CUDA(cudaMemsetAsync(b->p, 0, n * sizeof(double), d->stream));
    }
    S.alloc(S_NSLOTS);
    grid = std::min(d->lay.P * nc, 152 * 8);
    part.alloc((size_t)3 * grid);
    counter.alloc(1);
    TE_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), d->stream));
    TE_CUDA(cudaMemsetAsync(S.p, 0, S_NSLOTS * sizeof(double), d->stream));
    TE_CUDA(cudaMallocHost(&h, S_NSLOTS * sizeof(double)));
    TE_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    TE_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
    TE_CUDA(cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming));
  }
  ~KrylovWork() {
    for (auto& kv : graphs) {
      if (kv.second.x) cudaGraphExecDestroy(kv.second.x);
      if (kv.second.g) cudaGraphDestroy(kv.second.g);
    }
    if (h) cudaFreeHost(h);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (cap) cudaStreamDestroy(cap);
  }
  void read_scalars(cudaStream_t st) {
    TE_CUDA(cudaMemcpyAsync(h, S.p, S_NSLOTS * sizeof(double), cudaMemcpyDeviceToHost, st));
    TE_CUDA(cudaStreamSynchronize(st));
  }
};

static void launch_dots(KrylovWork& W, int nv, const double* a0, const double* b0, const double* a1, const double* b1,
                        const double* a2, const double* b2, int slot0, int fin, cudaStream_t st) {
  const Layout& L = W.d->lay;
  int npc = L.P * W.nc;
  if (nv == 1)
    k_dots<1><<<W.grid, KT, 0, st>>>(L, npc, a0, b0, a1, b1, a2, b2, W.part.p, W.counter.p, W.S.p, slot0, fin);
  else if (nv == 2)
    k_dots<2><<<W.grid, KT, 0, st>>>(L, npc, a0, b0, a1, b1, a2, b2, W.part.p, W.counter.p, W.S.p, slot0, fin);
  else
    k_dots<3><<<W.grid, KT, 0, st>>>(L, npc, a0, b0, a1, b1, a2, b2, W.part.p, W.counter.p, W.S.p, slot0, fin);
  count_launch();
  TE_LAUNCH_CHECK();
}

// one BiCGStab iteration (everything between two convergence tests)
static void iteration(KrylovWork& W, const te_operator* A, te_cycle* M, double* x, double tol, int flags,
                      cudaStream_t st) {
  const Layout& L = W.d->lay;
  int nc = W.nc, npc = L.P * nc;
  double* mp = M ? W.mp.p : W.p.p;
  double* ms = M ? W.ms.p : W.s.p;
  if (M) M->body(W.p.p, W.mp.p, st);
  operator_apply(A, nc, TE_F64, mp, W.ap.p, st);
  launch_dots(W, 1, W.rhat.p, W.ap.p, nullptr, nullptr, nullptr, nullptr, S_RHAT_AP, 1, st);
  k_s<<<W.grid, KT, 0, st>>>(L, npc, tol, W.resid.p, W.ap.p, W.s.p, W.part.p, W.counter.p, W.S.p);
  count_launch();
  TE_LAUNCH_CHECK();
  if (M) M->body(W.s.p, W.ms.p, st);
  operator_apply(A, nc, TE_F64, ms, W.as.p, st);
  launch_dots(W, 2, W.as.p, W.s.p, W.as.p, W.as.p, nullptr, nullptr, S_AS_S, 2, st);
  const double* dir = (M && (flags & TE_BICGSTAB_PRECONDITIONED_EXIT)) ? W.mp.p : W.p.p;
  k_xr<<<W.grid, KT, 0, st>>>(L, npc, x, W.resid.p, mp, ms, W.ap.p, W.as.p, W.rhat.p, dir, W.part.p,
                              W.counter.p, W.S.p);
  count_launch();
  TE_LAUNCH_CHECK();
  k_p<<<W.grid, KT, 0, st>>>(L, npc, W.p.p, W.ap.p, W.resid.p, W.S.p);
  count_launch();
  TE_LAUNCH_CHECK();
}

}  // namespace te

using namespace te;

extern "C" {

int te_bicgstab_solve(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* Mc, double tol,
                      int max_iterations, int flags, int* iterations, double* final_residual) {
  int status = TE_OK;
  int rc = guard([&] {
    require(A && xv && bv && iterations, "null argument");
    const te_domain* d = A->dom;
    cudaStream_t st = d->stream;
    // the solver's work vectors live with the operator (freed with it)
    auto& slot = A->krylov[nc];
    if (!slot) slot = std::make_shared<KrylovWork>(d, nc);
    KrylovWork& W = *std::static_pointer_cast<KrylovWork>(slot);
    te_cycle* M = const_cast<te_cycle*>(Mc);
    if (M) M->ensure(nc);
    double* x = (double*)xv;
    const double* b = (const double*)bv;
    size_t bytes = W.n * sizeof(double);
    // resid = b - A x; rhat = p = resid (BiCGStab.h:113-131)
    operator_apply(A, nc, TE_F64, x, W.resid.p, st);
    vec_dispatch(d, nc, TE_F64, OP_SCALE_THEN_ADD, W.resid.p, b, nullptr, -1, 0, 0);
    TE_CUDA(cudaMemcpyAsync(W.rhat.p, W.resid.p, bytes, cudaMemcpyDeviceToDevice, st));
    TE_CUDA(cudaMemcpyAsync(W.p.p, W.resid.p, bytes, cudaMemcpyDeviceToDevice, st));
    TE_CUDA(cudaMemsetAsync(W.S.p, 0, S_NSLOTS * sizeof(double), st));
    launch_dots(W, 3, b, b, W.rhat.p, W.resid.p, W.resid.p, W.resid.p, S_BB, 0, st);
    // S_BB, S_RHO? slots: S_BB = b.b, S_BB+1 and S_BB+2 are scratch; copy into place
    W.read_scalars(st);
    double bb = W.h[S_BB], rho = W.h[S_BB + 1], rr = W.h[S_BB + 2];
    double r0 = std::sqrt(bb);
    for (int i = 0; i < S_NSLOTS; i++) W.h[i] = 0.0;
    W.h[S_RHO] = rho;
    W.h[S_R0] = r0;
    TE_CUDA(cudaMemcpyAsync(W.S.p, W.h, S_NSLOTS * sizeof(double), cudaMemcpyHostToDevice, st));
    int its = 0;
    double residual = std::sqrt(rr) / r0;
    if (final_residual) *final_residual = residual;
    if (r0 == 0) {
      TE_CUDA(cudaStreamSynchronize(st));
      *iterations = 0;
      return;
    }
    const char* ng = getenv("TE_NO_GRAPH");
    bool use_graph = !(ng && ng[0] == '1');
    auto gkey = std::make_tuple((void*)x, (const void*)b, M ? M->serial : 0ull, M ? M->generation : 0ull, tol, flags);
    while (residual > tol && its < max_iterations) {
      if (rho == 0) {
        status = TE_ERR_BREAKDOWN;
        set_error("BiCGStab broke down, rho was 0 on iteration " + std::to_string(its));
        break;
      }
      if (use_graph) {
        auto it = W.graphs.find(gkey);
        if (it == W.graphs.end()) {
          KrylovWork::G g;
          long long l0 = g_launches.load();
          TE_CUDA(cudaStreamBeginCapture(W.cap, cudaStreamCaptureModeThreadLocal));
          try {
            iteration(W, A, M, x, tol, flags, W.cap);
          } catch (...) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(W.cap, &junk);
            if (junk) cudaGraphDestroy(junk);
            throw;
          }
          TE_CUDA(cudaStreamEndCapture(W.cap, &g.g));
          TE_CUDA(cudaGraphInstantiate(&g.x, g.g, 0));
          g.launches = g_launches.load() - l0;
          g_launches.fetch_sub(g.launches);
          it = W.graphs.emplace(gkey, g).first;
        }
        TE_CUDA(cudaEventRecord(W.ev_in, st));
        TE_CUDA(cudaStreamWaitEvent(W.cap, W.ev_in, 0));
        TE_CUDA(cudaGraphLaunch(it->second.x, W.cap));
        count_launch((int)it->second.launches);
        TE_CUDA(cudaEventRecord(W.ev_out, W.cap));
        TE_CUDA(cudaStreamWaitEvent(st, W.ev_out, 0));
      } else {
        iteration(W, A, M, x, tol, flags, st);
      }
      W.read_scalars(st);
      if (W.h[S_DONE] != 0.0) {  // ||s|| / ||b|| <= tol: x updated, stop (BiCGStab.h:162-168)
        if (final_residual) *final_residual = std::sqrt(W.h[S_SS]) / r0;
        break;
      }
      its++;
      rho = W.h[S_RHO];
      residual = std::sqrt(W.h[S_RR]) / r0;
      if (final_residual) *final_residual = residual;
    }
    *iterations = its;
  });
  return rc != TE_OK ? rc : status;
}

}  // extern "C"
