// Recording library calls into one CUDA graph (many trajectories / sizes per launch).
//
// l3es_graph_begin hands out a private capturing stream; every l3es_* call given that
// stream records its kernels instead of running them; l3es_graph_end instantiates the
// recorded work as one executable graph, launched with l3es_graph_launch on any
// stream. The graph keeps the device pointers it was recorded with.
#include <cuda_runtime.h>

#include <string>

#include "l3es_internal.h"

struct l3es_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

using namespace l3es;

extern "C" {

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
  auto* g = new l3es_graph();
  cudaError_t e = cudaStreamEndCapture(s, &g->graph);
  cudaStreamDestroy(s);
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
