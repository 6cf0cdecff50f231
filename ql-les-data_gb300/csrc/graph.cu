// Recording library calls into one CUDA graph (many trajectories / sizes per launch).
//
// l3es_graph_begin hands out a private capturing stream; every l3es_* call given that
// stream records its kernels instead of running them; l3es_graph_end instantiates the
// recorded work as one executable graph, launched with l3es_graph_launch on any
// stream. The graph keeps the device pointers it was recorded with.
//
// Branches: l3es_graph_fork opens a stream that joins the recording; its calls depend
// on what the recording held when it was opened and run concurrently with everything
// recorded elsewhere (other branches, later work on the capturing stream) until
// l3es_graph_join, after which the capturing stream's later work waits for it. Grids
// of different sizes in one recording then execute side by side instead of one after
// another. Branch streams live until l3es_graph_end.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "l3es_internal.h"

struct l3es_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

using namespace l3es;

namespace {
std::mutex g_branch_mu;
std::map<unsigned long long, std::vector<cudaStream_t>> g_branches;  // capture id -> branch streams

int capture_id(cudaStream_t s, unsigned long long* id, const char* who) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  int rc = cuda_check(cudaStreamGetCaptureInfo(s, &st, id), who);
  if (rc != L3ES_OK) return rc;
  if (st != cudaStreamCaptureStatusActive) return fail(L3ES_ESTATE, std::string(who) + ": stream is not recording");
  return L3ES_OK;
}

// one event record on `from` and a wait on `to`: `to` depends on what `from` holds now
int link(cudaStream_t from, cudaStream_t to, const char* who) {
  cudaEvent_t e = nullptr;
  int rc = cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), who);
  if (rc != L3ES_OK) return rc;
  rc = cuda_check(cudaEventRecord(e, from), who);
  if (rc == L3ES_OK) rc = cuda_check(cudaStreamWaitEvent(to, e, 0), who);
  cudaEventDestroy(e);
  return rc;
}
}  // namespace

extern "C" {

int l3es_graph_fork(void* capture_stream, void** branch_stream) {
  if (!capture_stream || !branch_stream) return fail(L3ES_EINVAL, "l3es_graph_fork: null argument");
  cudaStream_t s = (cudaStream_t)capture_stream;
  unsigned long long id = 0;
  int rc = capture_id(s, &id, "l3es_graph_fork");
  if (rc != L3ES_OK) return rc;
  cudaStream_t b = nullptr;
  rc = cuda_check(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking), "l3es_graph_fork: stream");
  if (rc != L3ES_OK) return rc;
  rc = link(s, b, "l3es_graph_fork");
  if (rc != L3ES_OK) {
    cudaStreamDestroy(b);
    return rc;
  }
  {
    std::lock_guard<std::mutex> lock(g_branch_mu);
    g_branches[id].push_back(b);
  }
  *branch_stream = (void*)b;
  return L3ES_OK;
}

int l3es_graph_join(void* capture_stream, void* branch_stream) {
  if (!capture_stream || !branch_stream) return fail(L3ES_EINVAL, "l3es_graph_join: null argument");
  return link((cudaStream_t)branch_stream, (cudaStream_t)capture_stream, "l3es_graph_join");
}

int l3es_graph_begin(void** capture_stream) {
  if (!capture_stream) return fail(L3ES_EINVAL, "l3es_graph_begin: null argument");
  cudaStream_t s = nullptr;
  int rc = cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "l3es_graph_begin: stream");
  if (rc != L3ES_OK) return rc;
  rc = cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "l3es_graph_begin: capture");
  if (rc != L3ES_OK) {
    cudaStreamDestroy(s);
    return rc;
  }
  *capture_stream = (void*)s;
  return L3ES_OK;
}

int l3es_graph_end(void* capture_stream, l3es_graph** out) {
  if (!capture_stream || !out) return fail(L3ES_EINVAL, "l3es_graph_end: null argument");
  *out = nullptr;
  cudaStream_t s = (cudaStream_t)capture_stream;
  unsigned long long id = 0;
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  const bool have_id = cudaStreamGetCaptureInfo(s, &st, &id) == cudaSuccess && st == cudaStreamCaptureStatusActive;
  auto* g = new l3es_graph();
  cudaError_t e = cudaStreamEndCapture(s, &g->graph);
  cudaStreamDestroy(s);
  if (have_id) {  // the recording's branch streams
    std::lock_guard<std::mutex> lock(g_branch_mu);
    auto it = g_branches.find(id);
    if (it != g_branches.end()) {
      for (cudaStream_t b : it->second) cudaStreamDestroy(b);
      g_branches.erase(it);
    }
  }
  if (e != cudaSuccess) {
    delete g;
    return cuda_check(e, "l3es_graph_end: capture");
  }
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g->graph);
    delete g;
    return cuda_check(e, "l3es_graph_end: instantiate");
  }
  *out = g;
  return L3ES_OK;
}

int l3es_graph_launch(l3es_graph* g, void* stream) {
  if (!g || !g->exec) return fail(L3ES_EINVAL, "l3es_graph_launch: null graph");
  return cuda_check(cudaGraphLaunch(g->exec, (cudaStream_t)stream), "l3es_graph_launch");
}

int l3es_graph_destroy(l3es_graph* g) {
  if (!g) return L3ES_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return L3ES_OK;
}

}  // extern "C"
