// chf_batch.cu -- an ensemble of independent channels stepped together.
//
// No counterpart in the reference (one channel per MPI job).  Small channels
// (32^3 .. 64 x 97 x 64) fill a GB300 poorly one at a time: each kernel of a
// step has a few dozen CTAs and the step is bound by launch latency.
//
// A batch holds n channels of any sizes, Reynolds numbers and precisions on
// one device.  Channels of the mixed precisions that share a grid (nnx, nny,
// nnz, product grid), time step, pressure gradient and box form a class, and
// a class is stepped as one stacked set of buffers: channel c of the class
// occupies spanwise slots c nny .. c nny + nny - 1 of a stacked field, so
// every kernel of the mixed step runs once for the whole class with the
// class's modes side by side (the z transforms and GEMMs over nch times the
// columns, the x/y transforms over nch times the planes, the curl and the
// solves over every channel's modes and k^2 groups, the (0,0) modes one per
// channel).  Per channel stay: the Reynolds number (the operator inverses and
// the explicit terms of its k^2 groups), the mean arrays and the flow-rate
// control.  A class is one ordinary handle inside the batch.  FP64 channels
// are stepped as themselves.
//
// Each channel also stays an ordinary chf_handle (lent by chf_batch_handle)
// for upload, download, diagnostics, statistics and restart files.
// chf_batch_step gathers the channels' states into their classes with one
// kernel per class, advances every class (pairs of steps replay one CUDA
// graph that forks into one branch per class or FP64 channel and joins
// back), and scatters the states back.  The per-column arithmetic of every
// kernel is that of a single channel, so each channel's results are
// bit-identical to stepping it alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

namespace {

constexpr int kMaxClass = 256;  // channels per class (pointer tables)

// Device pointer table of one class: the members' field slots, mean arrays
// and flow words (uploaded before each gather / scatter; the history swap
// moves the members' field pointers).
struct ClassTable {
  cd* f[F_COUNT][kMaxClass];
  double* mean[M_COUNT][kMaxClass];
  double* flow[kMaxClass];
};

struct Stack {
  chf_handle* h = nullptr;    // the stacked handle (owned by the batch)
  std::vector<int> members;   // channel indices, in slot order
  ClassTable* table = nullptr;  // device copy
  ClassTable host{};
};

}  // namespace

struct chf_batch {
  std::vector<chf_handle*> ch;
  std::vector<Stack> stacks;
  std::vector<int> solo;          // channels stepped as themselves (FP64)
  int device = 0;
  cudaStream_t stream = nullptr;  // the batch stream: gathers, graph launches, joins
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> ev_unit;  // one per stepping unit (class or FP64 channel)
  std::vector<cudaEvent_t> ev_ch;    // one per channel
  struct PairGraph {
    std::vector<cd*> f;           // every unit's history arrangement at capture
    cudaGraphExec_t exec;
  };
  std::vector<PairGraph> graphs;
  bool graphs_off = false;
  std::string err;
};

namespace {

bool ok(chf_batch* b, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  b->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

// the handles that step: the classes, then the FP64 channels
std::vector<chf_handle*> units(const chf_batch* b) {
  std::vector<chf_handle*> u;
  for (const auto& s : b->stacks) u.push_back(s.h);
  for (int i : b->solo) u.push_back(b->ch[i]);
  return u;
}

// ---------------------------------------------------------------------------
// Gather (dir = 0) / scatter (dir = 1) of one class, grid (blocks, nch):
// member c's field slots [n][chm] <-> spanwise block c of the stacked slots
// [n][nch chm]; its mean arrays <-> block c of the stacked [nch][2 NZ]; its
// flow word <-> block c of [nch][4].
// ---------------------------------------------------------------------------
__global__ void k_class_copy(const ClassTable* __restrict__ t, Ptr8<cd> sf, Ptr8<double> sm, double* sflow,
                             int NZ, long chm, int nch, int dir) {
  const int c = blockIdx.y;
  const long per = (long)NZ * chm;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < per; e += (long)gridDim.x * blockDim.x) {
    const long n = e / chm, m = e % chm;
    const size_t si = (size_t)n * nch * chm + (size_t)c * chm + m;
#pragma unroll
    for (int i = 0; i < F_COUNT; ++i) {
      cd* mf = t->f[i][c];
      if (dir == 0) sf.p[i][si] = mf[e];
      else mf[e] = sf.p[i][si];
    }
  }
  if (blockIdx.x == 0) {
    for (int k = threadIdx.x; k < 2 * NZ; k += blockDim.x)
      for (int i = 0; i < M_COUNT; ++i) {
        double* mm = t->mean[i][c];
        if (dir == 0) sm.p[i][(size_t)c * 2 * NZ + k] = mm[k];
        else mm[k] = sm.p[i][(size_t)c * 2 * NZ + k];
      }
    if (threadIdx.x < 4) {
      if (dir == 0) sflow[4 * c + threadIdx.x] = t->flow[c][threadIdx.x];
      else t->flow[c][threadIdx.x] = sflow[4 * c + threadIdx.x];
    }
  }
}

int class_copy(chf_batch* b, Stack& S, int dir) {
  chf_handle* h = S.h;
  const int nch = (int)S.members.size();
  for (int c = 0; c < nch; ++c) {
    const chf_handle* m = b->ch[S.members[c]];
    for (int i = 0; i < F_COUNT; ++i) S.host.f[i][c] = m->f[i];
    for (int i = 0; i < M_COUNT; ++i) S.host.mean[i][c] = m->mean[i];
    S.host.flow[c] = m->flow;
  }
  // pageable source: the copy is staged before the call returns
  if (!ok(b, cudaMemcpyAsync(S.table, &S.host, sizeof(ClassTable), cudaMemcpyHostToDevice, b->stream),
          "class table"))
    return CHF_E_CUDA;
  Ptr8<cd> sf{};
  Ptr8<double> sm{};
  for (int i = 0; i < F_COUNT; ++i) sf.p[i] = h->f[i];
  for (int i = 0; i < M_COUNT; ++i) sm.p[i] = h->mean[i];
  const long per = (long)h->d.NZ * h->d.chm;
  const unsigned blocks = (unsigned)std::min<long>((per + 255) / 256, 1024);
  k_class_copy<<<dim3(blocks, nch), 256, 0, b->stream>>>(S.table, sf, sm, h->flow, h->d.NZ, h->d.chm, nch, dir);
  return ok(b, cudaGetLastError(), "k_class_copy") ? CHF_OK : CHF_E_CUDA;
}

// ---------------------------------------------------------------------------
// A class's stacked handle, built from its members' handles: their operator
// inverses (and, for CHF_MIXED, increment operators) side by side, k^2
// groups with per-group Reynolds numbers, the (0,0) groups after them; the
// tensor-core plans and buffers of the stacked width (setup_mixed).
// ---------------------------------------------------------------------------
template <typename T>
bool dup(chf_batch* b, T** dst, const T* src, size_t count, const char* what) {
  return ok(b, cudaMalloc((void**)dst, sizeof(T) * count), what) &&
         ok(b, cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyDeviceToDevice), what);
}

int build_stack(chf_batch* b, Stack& S) {
  const int nch = (int)S.members.size();
  const Handle& c0 = *b->ch[S.members[0]];
  chf_handle* h = new (std::nothrow) chf_handle();
  if (!h) return CHF_E_NOMEM;
  S.h = h;
  h->cfg = c0.cfg;
  h->tune = c0.tune;
  h->device = c0.device;
  h->num_sms = c0.num_sms;
  h->prof.resize(K_COUNT);
  for (int k = 0; k < K_COUNT; ++k) h->prof[k] = {kKernelNames[k], 0, 0.0};
  Dims& d = h->d;
  d = c0.d;
  d.KY = c0.d.KY * nch;
  d.nch = nch;
  d.chm = c0.d.modes();
  const int NZ = d.NZ;
  if (!ok(b, cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking), "cudaStreamCreate"))
    return CHF_E_CUDA;
  h->stream = h->own_stream;
  const size_t fe = d.field_elems();
  for (int i = 0; i < F_COUNT; ++i)
    if (!ok(b, cudaMalloc((void**)&h->f[i], sizeof(cd) * fe), "class state")) return CHF_E_NOMEM;
  for (int i = 0; i < M_COUNT; ++i)
    if (!ok(b, cudaMalloc((void**)&h->mean[i], sizeof(double) * 2 * NZ * nch), "class means")) return CHF_E_NOMEM;
  if (!ok(b, cudaMalloc((void**)&h->dev_status, sizeof(int)), "class status") ||
      !ok(b, cudaMemset(h->dev_status, 0, sizeof(int)), "class status") ||
      !ok(b, cudaMalloc((void**)&S.table, sizeof(ClassTable)), "class table"))
    return CHF_E_NOMEM;
  // wavenumbers: iapha as the members', ibeta repeated per channel
  if (!dup(b, &h->iapha, c0.iapha, d.KX, "class iapha")) return CHF_E_CUDA;
  if (!ok(b, cudaMalloc((void**)&h->ibeta, sizeof(double) * d.KY), "class ibeta")) return CHF_E_NOMEM;
  for (int c = 0; c < nch; ++c)
    if (!ok(b, cudaMemcpy(h->ibeta + (size_t)c * c0.d.KY, c0.ibeta, sizeof(double) * c0.d.KY,
                          cudaMemcpyDeviceToDevice), "class ibeta"))
      return CHF_E_CUDA;
  // FFT plans and twiddles of the members' lengths
  h->py = c0.py;
  h->px = c0.px;
  h->py64 = c0.py64;
  h->px64 = c0.px64;
  if (upload_stage_twiddles(h) != CHF_OK) {
    b->err = "class set-up: " + h->err;
    return CHF_E_CUDA;
  }
  h->pz2 = c0.pz2;
  h->pzm = c0.pzm;
  if (!dup(b, &h->tw_py, c0.tw_py, c0.d.PY, "class twiddles") || !dup(b, &h->tw_px, c0.tw_px, c0.d.PX, "class twiddles") ||
      !dup(b, &h->tw_z2, c0.tw_z2, 2 * c0.d.N, "class twiddles") ||
      !dup(b, &h->tw_zm, c0.tw_zm, 2 * c0.d.MZ, "class twiddles"))
    return CHF_E_CUDA;
  // k^2 groups of every member side by side, then the members' (0,0) groups
  h->sl = c0.sl;
  const size_t stride = h->sl.stride;
  std::vector<double> k2v, gre;
  std::vector<int> gstart, gmodes;
  std::vector<size_t> goff(nch);
  for (int c = 0; c < nch; ++c) {
    const Handle& m = *b->ch[S.members[c]];
    std::vector<int> st(m.nk2 + 1), md(std::max(1, m.nsolve));
    std::vector<double> kv(m.nk2 + 1);
    if (!ok(b, cudaMemcpy(st.data(), m.group_start, sizeof(int) * st.size(), cudaMemcpyDeviceToHost), "groups") ||
        !ok(b, cudaMemcpy(md.data(), m.group_modes, sizeof(int) * md.size(), cudaMemcpyDeviceToHost), "groups") ||
        !ok(b, cudaMemcpy(kv.data(), m.k2vals, sizeof(double) * kv.size(), cudaMemcpyDeviceToHost), "groups"))
      return CHF_E_CUDA;
    goff[c] = k2v.size();
    for (int g = 0; g < m.nk2; ++g) {
      gstart.push_back((int)gmodes.size());
      k2v.push_back(kv[g]);
      gre.push_back(m.cfg.re);
      for (int q = st[g]; q < st[g + 1]; ++q) gmodes.push_back(md[q] + (int)(c * d.chm));
    }
  }
  h->nk2 = (int)k2v.size();
  h->nsolve = (int)gmodes.size();
  gstart.push_back((int)gmodes.size());
  for (int c = 0; c < nch; ++c) {
    k2v.push_back(0.0);
    gre.push_back(b->ch[S.members[c]]->cfg.re);
  }
  auto up = [b](auto** dst, const auto& v, const char* what) {
    using E = typename std::decay<decltype(v[0])>::type;
    return ok(b, cudaMalloc((void**)dst, sizeof(E) * std::max<size_t>(1, v.size())), what) &&
           ok(b, cudaMemcpy(*dst, v.data(), sizeof(E) * v.size(), cudaMemcpyHostToDevice), what);
  };
  if (!up(&h->k2vals, k2v, "class k2") || !up(&h->group_start, gstart, "class groups") ||
      !up(&h->group_modes, gmodes, "class groups") || !up(&h->group_re, gre, "class re"))
    return CHF_E_CUDA;
  if (!ok(b, cudaMalloc((void**)&h->xinv, sizeof(double) * stride * (size_t)(h->nk2 + nch)), "class inverses"))
    return CHF_E_NOMEM;
  for (int c = 0; c < nch; ++c) {
    const Handle& m = *b->ch[S.members[c]];
    if (!ok(b, cudaMemcpy(h->xinv + goff[c] * stride, m.xinv, sizeof(double) * stride * m.nk2,
                          cudaMemcpyDeviceToDevice), "class inverses") ||
        !ok(b, cudaMemcpy(h->xinv + (size_t)(h->nk2 + c) * stride, m.xinv + (size_t)m.nk2 * stride,
                          sizeof(double) * stride, cudaMemcpyDeviceToDevice), "class inverses"))
      return CHF_E_CUDA;
  }
  // constant flow rate per channel
  std::vector<double> ubp(nch);
  if (!ok(b, cudaMalloc((void**)&h->phi, sizeof(double) * NZ * nch), "class phi") ||
      !ok(b, cudaMalloc((void**)&h->flow, sizeof(double) * 4 * nch), "class flow"))
    return CHF_E_NOMEM;
  for (int c = 0; c < nch; ++c) {
    const Handle& m = *b->ch[S.members[c]];
    ubp[c] = m.ubphi;
    if (!ok(b, cudaMemcpy(h->phi + (size_t)c * NZ, m.phi, sizeof(double) * NZ, cudaMemcpyDeviceToDevice), "class phi"))
      return CHF_E_CUDA;
  }
  if (!up(&h->ubphi_dev, ubp, "class phi")) return CHF_E_CUDA;
  // the mixed nonlinear term over the stacked columns
  int rc = setup_mixed(h);
  if (rc != CHF_OK) {
    b->err = "class set-up: " + h->err;
    return rc;
  }
  if (increment_solve(h) && h->nk2 > 0) {
    if (!ok(b, cudaMalloc((void**)&h->incm, sizeof(float2) * stride * h->nk2), "class increment operators") ||
        !ok(b, cudaMalloc((void**)&h->incx, sizeof(float) * stride * h->nk2), "class increment operators") ||
        !ok(b, cudaMalloc((void**)&h->incr_exp, (size_t)2 * NZ * h->nk2), "class increment operators"))
      return CHF_E_NOMEM;
    for (int c = 0; c < nch; ++c) {
      const Handle& m = *b->ch[S.members[c]];
      if (m.nk2 == 0) continue;
      if (!ok(b, cudaMemcpy(h->incm + goff[c] * stride, m.incm, sizeof(float2) * stride * m.nk2,
                            cudaMemcpyDeviceToDevice), "class increment operators") ||
          !ok(b, cudaMemcpy(h->incx + goff[c] * stride, m.incx, sizeof(float) * stride * m.nk2,
                            cudaMemcpyDeviceToDevice), "class increment operators") ||
          !ok(b, cudaMemcpy(h->incr_exp + goff[c] * 2 * NZ, m.incr_exp, (size_t)2 * NZ * m.nk2,
                            cudaMemcpyDeviceToDevice), "class increment operators"))
        return CHF_E_CUDA;
    }
    h->rec_df_rule = c0.rec_df_rule;  // the members' arithmetic
    if (setup_inc_items(h) != CHF_OK) {
      b->err = "class set-up: " + h->err;
      return CHF_E_CUDA;
    }
    if (!ok(b, cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !ok(b, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming), "cudaEventCreate") ||
        !ok(b, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming), "cudaEventCreate"))
      return CHF_E_CUDA;
  }
  h->kernels_per_step = c0.kernels_per_step;
  h->uploaded = true;
  return ok(b, cudaDeviceSynchronize(), "class set-up") ? CHF_OK : CHF_E_CUDA;
}

void arrangement(const chf_batch* b, std::vector<cd*>* f) {
  f->clear();
  for (auto* h : units(b)) f->insert(f->end(), h->f, h->f + F_COUNT);
}

void restore(chf_batch* b, const std::vector<cd*>& f) {
  const auto u = units(b);
  for (size_t i = 0; i < u.size(); ++i) std::memcpy(u[i]->f, f.data() + i * F_COUNT, sizeof(cd*) * F_COUNT);
}

// fork: every unit stream waits for the batch stream
bool fork_all(chf_batch* b) {
  if (!ok(b, cudaEventRecord(b->fork, b->stream), "batch fork")) return false;
  for (auto* h : units(b))
    if (!ok(b, cudaStreamWaitEvent(h->stream, b->fork, 0), "batch fork")) return false;
  return true;
}

// join: the batch stream waits for every unit stream
bool join_all(chf_batch* b) {
  const auto u = units(b);
  for (size_t i = 0; i < u.size(); ++i)
    if (!ok(b, cudaEventRecord(b->ev_unit[i], u[i]->stream), "batch join") ||
        !ok(b, cudaStreamWaitEvent(b->stream, b->ev_unit[i], 0), "batch join"))
      return false;
  return true;
}

int step_all(chf_batch* b, int steps) {
  for (auto* h : units(b))
    for (int s = 0; s < steps; ++s) {
      int rc = step_once(h);
      if (rc != CHF_OK) {
        b->err = "channel step: " + h->err;
        return rc;
      }
    }
  return CHF_OK;
}

// the two-step graph for the current arrangements (nullptr: step directly)
int pair_graph(chf_batch* b, cudaGraphExec_t* out) {
  *out = nullptr;
  if (b->graphs_off) return CHF_OK;
  for (auto* h : b->ch)
    if (h->profiling) return CHF_OK;
  std::vector<cd*> f;
  arrangement(b, &f);
  for (auto& g : b->graphs)
    if (g.f == f) {
      *out = g.exec;
      return CHF_OK;
    }
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    b->graphs_off = true;
    return CHF_OK;
  }
  int rc = fork_all(b) ? step_all(b, 2) : CHF_E_CUDA;
  if (rc == CHF_OK && !join_all(b)) rc = CHF_E_CUDA;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  chf_batch::PairGraph pg{f, nullptr};
  const bool good = rc == CHF_OK && e == cudaSuccess && graph &&
                    cudaGraphInstantiate(&pg.exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  restore(b, f);  // the captured launches did not run
  if (!good) {
    cudaGetLastError();
    b->err.clear();
    b->graphs_off = true;
    return CHF_OK;
  }
  b->graphs.push_back(pg);
  *out = pg.exec;
  return CHF_OK;
}

void release(chf_batch* b) {
  cudaSetDevice(b->device);
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  for (auto e : b->ev_unit) cudaEventDestroy(e);
  for (auto e : b->ev_ch) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->done) cudaEventDestroy(b->done);
  if (b->stream) cudaStreamDestroy(b->stream);
  for (auto& s : b->stacks) {
    if (s.table) cudaFree(s.table);
    if (s.h) chf_destroy(s.h);
  }
  for (auto* h : b->ch) chf_destroy(h);
}

thread_local std::string g_batch_create_error;

int create_fail(chf_batch* b, int rc, const std::string& why) {
  g_batch_create_error = why;
  release(b);
  delete b;
  return rc;
}

}  // namespace

extern "C" {

int chf_batch_create(int n, const chf_config* cfgs, chf_batch** out) {
  if (!out || n < 1 || !cfgs) {
    g_batch_create_error = "n must be >= 1 and cfgs, out non-NULL";
    return CHF_E_INVALID;
  }
  *out = nullptr;
  for (int i = 1; i < n; ++i)
    if (cfgs[i].device != cfgs[0].device) {
      g_batch_create_error = "all channels of a batch must be on one device";
      return CHF_E_INVALID;
    }
  chf_batch* b = new (std::nothrow) chf_batch();
  if (!b) return CHF_E_NOMEM;
  b->device = cfgs[0].device;
  for (int i = 0; i < n; ++i) {
    chf_handle* h = nullptr;
    int rc = chf_create(&cfgs[i], &h);
    if (rc != CHF_OK) return create_fail(b, rc, "channel " + std::to_string(i) + ": " + chf_last_error(nullptr));
    b->ch.push_back(h);
  }
  if (!ok(b, cudaSetDevice(b->device), "cudaSetDevice") ||
      !ok(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !ok(b, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate") ||
      !ok(b, cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "cudaEventCreate"))
    return create_fail(b, CHF_E_CUDA, b->err);
  // classes: mixed-precision channels of one grid, time step, pressure
  // gradient and box, in the order of their first member
  std::map<std::tuple<int, int, int, int, int, double, double, double, double>, int> cls;
  for (int i = 0; i < n; ++i) {
    const Handle& h = *b->ch[i];
    if (!mixed_front(&h)) {
      b->solo.push_back(i);
      continue;
    }
    const auto key = std::make_tuple(h.d.nnx, h.d.nny, h.d.nnz, h.d.MZ, h.cfg.precision, h.cfg.dt, h.cfg.re_p,
                                     h.cfg.aphi, h.cfg.beta);
    auto it = cls.find(key);
    if (it == cls.end() || (int)b->stacks[it->second].members.size() == kMaxClass) {
      cls[key] = (int)b->stacks.size();
      b->stacks.emplace_back();
      it = cls.find(key);
    }
    b->stacks[it->second].members.push_back(i);
  }
  for (auto& s : b->stacks) {
    const int rc = build_stack(b, s);
    if (rc != CHF_OK) return create_fail(b, rc, b->err.empty() ? "class set-up failed" : b->err);
  }
  b->ev_unit.resize(units(b).size(), nullptr);
  b->ev_ch.resize(n, nullptr);
  for (auto* v : {&b->ev_unit, &b->ev_ch})
    for (auto& e : *v)
      if (!ok(b, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate"))
        return create_fail(b, CHF_E_CUDA, b->err);
  *out = b;
  return CHF_OK;
}

int chf_batch_destroy(chf_batch* b) {
  if (!b) return CHF_E_INVALID;
  release(b);
  delete b;
  return CHF_OK;
}

const char* chf_batch_last_error(const chf_batch* b) {
  return b ? b->err.c_str() : g_batch_create_error.c_str();
}

int chf_batch_size(const chf_batch* b) { return b ? (int)b->ch.size() : 0; }

int chf_batch_handle(chf_batch* b, int i, chf_handle** h) {
  if (!b || !h || i < 0 || i >= (int)b->ch.size()) return CHF_E_INVALID;
  *h = b->ch[i];
  return CHF_OK;
}

int chf_batch_step(chf_batch* b, int nsteps) {
  if (!b) return CHF_E_INVALID;
  if (nsteps < 0) {
    b->err = "nsteps must be >= 0";
    return CHF_E_INVALID;
  }
  for (size_t i = 0; i < b->ch.size(); ++i)
    if (!b->ch[i]->uploaded) {
      b->err = "channel " + std::to_string(i) + " has no state (chf_upload_state)";
      return CHF_E_STATE;
    }
  if (!ok(b, cudaSetDevice(b->device), "cudaSetDevice")) return CHF_E_CUDA;
  if (nsteps == 0) return CHF_OK;
  // the batch stream waits for work already queued on the channels' streams
  for (size_t i = 0; i < b->ch.size(); ++i)
    if (!ok(b, cudaEventRecord(b->ev_ch[i], b->ch[i]->stream), "batch order") ||
        !ok(b, cudaStreamWaitEvent(b->stream, b->ev_ch[i], 0), "batch order"))
      return CHF_E_CUDA;
  for (auto& s : b->stacks) {
    const int rc = class_copy(b, s, 0);
    if (rc != CHF_OK) return rc;
  }
  int s = 0;
  if (nsteps >= 2) {
    cudaGraphExec_t g = nullptr;
    int rc = pair_graph(b, &g);
    if (rc != CHF_OK) return rc;
    if (g)
      for (; s + 2 <= nsteps; s += 2)
        if (!ok(b, cudaGraphLaunch(g, b->stream), "cudaGraphLaunch")) return CHF_E_CUDA;
  }
  if (s < nsteps) {
    if (!fork_all(b)) return CHF_E_CUDA;
    int rc = step_all(b, nsteps - s);
    if (rc != CHF_OK) return rc;
    if (!join_all(b)) return CHF_E_CUDA;
  }
  // the classes' history swaps leave their field slots in some arrangement;
  // the scatter copies slot by slot into the members' current slots
  for (auto& st : b->stacks) {
    const int rc = class_copy(b, st, 1);
    if (rc != CHF_OK) return rc;
  }
  // later work on a channel stream (download, diagnostics) waits for the batch
  if (!ok(b, cudaEventRecord(b->done, b->stream), "batch done")) return CHF_E_CUDA;
  for (auto* h : b->ch)
    if (!ok(b, cudaStreamWaitEvent(h->stream, b->done, 0), "batch done")) return CHF_E_CUDA;
  return CHF_OK;
}

int chf_batch_synchronize(chf_batch* b) {
  if (!b) return CHF_E_INVALID;
  if (!ok(b, cudaSetDevice(b->device), "cudaSetDevice") ||
      !ok(b, cudaStreamSynchronize(b->stream), "cudaStreamSynchronize"))
    return CHF_E_CUDA;
  for (size_t i = 0; i < b->ch.size(); ++i) {
    int rc = chf_synchronize(b->ch[i]);
    if (rc != CHF_OK) {
      b->err = "channel " + std::to_string(i) + ": " + b->ch[i]->err;
      return rc;
    }
  }
  for (auto& s : b->stacks) {
    int rc = chf_synchronize(s.h);
    if (rc != CHF_OK) {
      b->err = "class: " + s.h->err;
      return rc;
    }
  }
  return CHF_OK;
}

}  // extern "C"
