// chf_batch.cu -- an ensemble of independent channels stepped together.
//
// No counterpart in the reference (one channel per MPI job).  Small channels
// (32^3 .. 64 x 97 x 64) fill a GB300 poorly one at a time: their kernels
// have a few dozen CTAs and a step is bound by launch latency.  A batch
// holds n channels of any sizes, Reynolds numbers and precisions on one
// device and advances all of them with one CUDA-graph launch per pair of
// steps.  The graph forks from the batch stream into one branch per channel
// (the channel's own stream) and joins back, so the channels' kernels run
// side by side on the SMs.  Each channel stays an ordinary chf_handle
// (borrowed through chf_batch_handle) for upload, download, diagnostics and
// restart files; its results are bit-identical to stepping it alone.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

struct chf_batch {
  std::vector<chf_handle*> ch;
  int device = 0;
  cudaStream_t stream = nullptr;  // the batch stream: graph launches and joins
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> ev;    // one per channel
  struct PairGraph {
    std::vector<cd*> f;           // every channel's history arrangement at capture
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

void arrangement(const chf_batch* b, std::vector<cd*>* f) {
  f->clear();
  for (auto* h : b->ch) f->insert(f->end(), h->f, h->f + F_COUNT);
}

void restore(chf_batch* b, const std::vector<cd*>& f) {
  for (size_t i = 0; i < b->ch.size(); ++i) std::memcpy(b->ch[i]->f, f.data() + i * F_COUNT, sizeof(cd*) * F_COUNT);
}

// fork: every channel stream waits for the batch stream
bool fork_all(chf_batch* b) {
  if (!ok(b, cudaEventRecord(b->fork, b->stream), "batch fork")) return false;
  for (auto* h : b->ch)
    if (!ok(b, cudaStreamWaitEvent(h->stream, b->fork, 0), "batch fork")) return false;
  return true;
}

// join: the batch stream waits for every channel stream
bool join_all(chf_batch* b) {
  for (size_t i = 0; i < b->ch.size(); ++i)
    if (!ok(b, cudaEventRecord(b->ev[i], b->ch[i]->stream), "batch join") ||
        !ok(b, cudaStreamWaitEvent(b->stream, b->ev[i], 0), "batch join"))
      return false;
  return true;
}

int step_all(chf_batch* b, int steps) {
  for (auto* h : b->ch)
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
  for (auto e : b->ev) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->done) cudaEventDestroy(b->done);
  if (b->stream) cudaStreamDestroy(b->stream);
  for (auto* h : b->ch) chf_destroy(h);
}

thread_local std::string g_batch_create_error;

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
    if (rc != CHF_OK) {
      g_batch_create_error = "channel " + std::to_string(i) + ": " + chf_last_error(nullptr);
      release(b);
      delete b;
      return rc;
    }
    b->ch.push_back(h);
  }
  if (!ok(b, cudaSetDevice(b->device), "cudaSetDevice") ||
      !ok(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !ok(b, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate") ||
      !ok(b, cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "cudaEventCreate")) {
    g_batch_create_error = b->err;
    release(b);
    delete b;
    return CHF_E_CUDA;
  }
  b->ev.resize(n, nullptr);
  for (int i = 0; i < n; ++i)
    if (!ok(b, cudaEventCreateWithFlags(&b->ev[i], cudaEventDisableTiming), "cudaEventCreate")) {
      g_batch_create_error = b->err;
      release(b);
      delete b;
      return CHF_E_CUDA;
    }
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
  // the batch stream waits for work already queued on the channel streams
  if (!join_all(b)) return CHF_E_CUDA;
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
  return CHF_OK;
}

}  // extern "C"
