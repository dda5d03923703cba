// api.cu — context, status reporting, CUDA-graph capture and test hooks of
// the C ABI.  The reference reports errors by aborting (SErr -> assert,
// debug.hpp:60-69); every entry point here returns a status instead and
// keeps a per-context message.
#include <cstdarg>
#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace flg {

int set_error(flg_ctx ctx, int code, const char *fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return code;
}

int cuda_fail(flg_ctx ctx, cudaError_t e, const char *what) {
  int code = e == cudaErrorMemoryAllocation ? FLG_ERR_OOM : FLG_ERR_CUDA;
  if (e == cudaErrorStreamCaptureUnsupported || e == cudaErrorStreamCaptureInvalidated) code = FLG_ERR_STATE;
  return set_error(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

__global__ void k_wait_unset(const uint32_t *word, uint32_t limit, uint32_t *err) {
  wait_flag(word, 0xFFFFFFFFu, limit, err);
}

}  // namespace flg

using namespace flg;

static constexpr uint32_t kDefaultSpinLimit = 1u << 22;

FLG_API const char *flg_version(void) { return "fledge-gb300 0.1 (sm_103a)"; }

FLG_API const char *flg_status_string(int s) {
  switch (s) {
    case FLG_OK: return "ok";
    case FLG_ERR_ARG: return "invalid argument";
    case FLG_ERR_OOM: return "out of memory";
    case FLG_ERR_CUDA: return "CUDA error";
    case FLG_ERR_TIMEOUT: return "device wait timed out";
    case FLG_ERR_STACK: return "traversal stack overflow";
    case FLG_ERR_STATE: return "invalid state";
    case FLG_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

FLG_API int flg_ctx_create(int32_t device, void *stream, flg_ctx *out) {
  if (!out) return FLG_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return FLG_ERR_CUDA;
  }
  if (device < 0 || device >= n) return FLG_ERR_ARG;
  flg_ctx c = new flg_ctx_t();
  c->device = device;
  c->spin_limit = kDefaultSpinLimit;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) {
    if (stream) {
      c->stream = (cudaStream_t)stream;
    } else {
      e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
      c->own_stream = true;
    }
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&c->d_err, 2 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, 2 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMallocHost((void **)&c->h_err, sizeof(uint32_t));
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&c->ev[k], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cudaGetLastError();
    flg_ctx_destroy(c);
    return e == cudaErrorMemoryAllocation ? FLG_ERR_OOM : FLG_ERR_CUDA;
  }
  *out = c;
  return FLG_OK;
}

FLG_API int flg_ctx_destroy(flg_ctx c) {
  if (!c) return FLG_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  for (int k = 0; k < 4; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  cudaFree(c->d_err);
  if (c->h_err) cudaFreeHost(c->h_err);
  cudaFree(c->d_ovf);
  cudaFree(c->d_ovf_count);
  cudaFree(c->d_work);
  cudaFree(c->d_ray_off);
  cudaFree(c->stage);
  cudaFree(c->pt_buf);
  cudaFree(c->rs_buf);
  for (cudaEvent_t e : c->stage_pool) cudaEventDestroy(e);
  delete c;
  return FLG_OK;
}

FLG_API int flg_ctx_set_stage_timing(flg_ctx c, int32_t on) {
  if (!c) return FLG_ERR_ARG;
  c->stage_timing = on != 0;
  c->stage_marks.clear();
  return FLG_OK;
}

FLG_API int flg_ctx_stage_times(flg_ctx c, char *json, size_t len) {
  if (!c || !json || len == 0) return c ? set_error(c, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  json[0] = 0;
  // per stage name (first-seen order): summed milliseconds and count
  std::vector<const char *> names;
  std::vector<double> ms;
  std::vector<int64_t> cnt;
  if (!c->stage_marks.empty()) {
    FLG_CUDA(c, cudaEventSynchronize(c->stage_marks.back().second));
    for (size_t k = 1; k < c->stage_marks.size(); ++k) {
      const char *nm = c->stage_marks[k].first;
      if (std::string(nm) == "start") continue;
      float t = 0.0f;
      FLG_CUDA(c, cudaEventElapsedTime(&t, c->stage_marks[k - 1].second, c->stage_marks[k].second));
      size_t j = 0;
      while (j < names.size() && std::string(names[j]) != nm) ++j;
      if (j == names.size()) {
        names.push_back(nm);
        ms.push_back(0.0);
        cnt.push_back(0);
      }
      ms[j] += t;
      cnt[j] += 1;
    }
  }
  std::string out = "{";
  char buf[160];
  for (size_t j = 0; j < names.size(); ++j) {
    snprintf(buf, sizeof buf, "%s\"%s\": {\"ms\": %.6f, \"n\": %lld}", j ? ", " : "", names[j], ms[j],
             (long long)cnt[j]);
    out += buf;
  }
  out += "}";
  c->stage_marks.clear();
  if (out.size() + 1 > len) return set_error(c, FLG_ERR_ARG, "stage-time buffer too small (%zu bytes needed)",
                                             out.size() + 1);
  memcpy(json, out.c_str(), out.size() + 1);
  return FLG_OK;
}

FLG_API void *flg_ctx_stream(flg_ctx c) { return c ? (void *)c->stream : nullptr; }

FLG_API int64_t flg_ctx_launch_count(flg_ctx c) { return c ? c->launches : 0; }

FLG_API int flg_ctx_set_spin_limit(flg_ctx c, uint32_t spins) {
  if (!c) return FLG_ERR_ARG;
  c->spin_limit = spins ? spins : kDefaultSpinLimit;
  return FLG_OK;
}

FLG_API int flg_ctx_last_error(flg_ctx c, char *buf, size_t len) {
  if (!c || !buf || !len) return FLG_ERR_ARG;
  std::strncpy(buf, c->last_error.c_str(), len - 1);
  buf[len - 1] = '\0';
  return FLG_OK;
}

FLG_API int flg_ctx_sync(flg_ctx c) {
  if (!c) return FLG_ERR_ARG;
  if (c->capturing) return set_error(c, FLG_ERR_STATE, "sync during capture");
  FLG_CUDA(c, cudaStreamSynchronize(c->copy_stream));
  FLG_CUDA(c, cudaStreamSynchronize(c->stream));
  FLG_CUDA(c, cudaMemcpy(c->h_err, c->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  const uint32_t e = *c->h_err;
  if (e) {
    FLG_CUDA(c, cudaMemset(c->d_err, 0, sizeof(uint32_t)));
    if (e & kErrTimeout) return set_error(c, FLG_ERR_TIMEOUT, "a bounded device-side wait timed out");
    if (e & kErrStack) return set_error(c, FLG_ERR_STACK, "traversal stack overflow");
    if (e & kErrQueue) return set_error(c, FLG_ERR_STATE, "wide-node work queue overflow");
  }
  return FLG_OK;
}

FLG_API int flg_debug_wait_unset_flag(flg_ctx c, uint32_t spins) {
  if (!c) return FLG_ERR_ARG;
  k_wait_unset<<<1, 1, 0, c->stream>>>(c->d_err + 1, spins, c->d_err);
  FLG_LAUNCH_CHECK(c, "k_wait_unset");
  return flg_ctx_sync(c);
}

FLG_API int flg_graph_begin(flg_ctx c) {
  if (!c) return FLG_ERR_ARG;
  if (c->capturing) return set_error(c, FLG_ERR_STATE, "capture already in progress");
  FLG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  c->capturing = true;
  return FLG_OK;
}

FLG_API int flg_graph_end(flg_ctx c, flg_graph *out) {
  if (!c || !out) return FLG_ERR_ARG;
  *out = nullptr;
  if (!c->capturing) return set_error(c, FLG_ERR_STATE, "no capture in progress");
  c->capturing = false;
  flg_graph g = new flg_graph_t();
  cudaError_t e = cudaStreamEndCapture(c->stream, &g->graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(c, e, "graph capture");
  }
  *out = g;
  return FLG_OK;
}

FLG_API int flg_graph_launch(flg_ctx c, flg_graph g) {
  if (!c || !g) return FLG_ERR_ARG;
  FLG_CUDA(c, cudaGraphLaunch(g->exec, c->stream));
  return FLG_OK;
}

FLG_API int flg_graph_destroy(flg_graph g) {
  if (!g) return FLG_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return FLG_OK;
}
