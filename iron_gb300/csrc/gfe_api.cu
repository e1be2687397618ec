// gfe_api.cu -- library-level entry points: version, error text, device error word, scratch.
#include <mutex>
#include <string>

#include "gfe_internal.cuh"

namespace {
thread_local std::string t_last_error;
thread_local unsigned* t_err_word = nullptr;  // gfe_set_thread_error_word override
std::mutex g_mu;
unsigned* g_err_word[64] = {nullptr};
int g_sm_count[64] = {0};
bool g_pool_ready[64] = {false};
// Freed stream-ordered scratch the device's default memory pool keeps mapped for the next call
// (the pool's release threshold; the default of 0 unmaps it at every synchronisation, so each
// Jacobian or Krylov solve would map its gigabytes of scratch again).  A process setting: it ends
// with the process.
constexpr uint64_t kScratchCacheBytes = 4ull << 30;

void prepare_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_pool_ready[dev]) return;
  g_pool_ready[dev] = true;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = kScratchCacheBytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
}
}  // namespace

namespace gfe {

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  // the failure is reported by this return code: clear the CUDA runtime's per-thread error state,
  // so a later launch check on this thread does not report it again as its own
  cudaGetLastError();
  return code;
}

unsigned* device_error_word() {
  if (t_err_word) return t_err_word;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_err_word[dev]) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(unsigned)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(unsigned)) != cudaSuccess) return nullptr;
    g_err_word[dev] = static_cast<unsigned*>(p);
  }
  return g_err_word[dev];
}

unsigned* thread_error_word() { return t_err_word; }
void set_thread_error_word(unsigned* w) { t_err_word = w; }

int scratch_alloc(void** p, size_t bytes, cudaStream_t s, const char* what) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  prepare_pool();
  cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(GFE_ERR_NOMEM, "device scratch for %s (%zu bytes) could not be allocated: %s", what, bytes,
                     cudaGetErrorString(e));
  }
  return GFE_OK;
}

void scratch_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

int sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!g_sm_count[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    g_sm_count[dev] = n > 0 ? n : 148;
  }
  return g_sm_count[dev];
}

}  // namespace gfe

extern "C" int gfe_version(void) { return 100; }

extern "C" int gfe_clear_stale_error(void) { return (int)cudaGetLastError(); }

extern "C" int gfe_release_scratch(void) {
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  cudaMemPool_t pool;
  GFE_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
  GFE_CUDA_TRY(cudaDeviceSynchronize());
  GFE_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
  return GFE_OK;
}

extern "C" int gfe_last_error(char* buf, int len) {
  int n = (int)t_last_error.size();
  if (buf && len > 0) {
    int k = n < len - 1 ? n : len - 1;
    for (int i = 0; i < k; ++i) buf[i] = t_last_error[i];
    buf[k] = 0;
  }
  return n;
}

extern "C" int gfe_set_thread_error_word(uint32_t* dev_word) {
  if (dev_word && (reinterpret_cast<uintptr_t>(dev_word) & 3))
    return gfe::set_error(GFE_ERR_ARG, "gfe_set_thread_error_word: word must be 4-byte aligned");
  t_err_word = reinterpret_cast<unsigned*>(dev_word);
  return GFE_OK;
}

extern "C" int gfe_device_errors(uint32_t* bits_host, void* stream) {
  if (!bits_host) return gfe::set_error(GFE_ERR_ARG, "gfe_device_errors: bits_host is NULL");
  unsigned* w = gfe::device_error_word();
  if (!w) return gfe::set_error(GFE_ERR_CUDA, "gfe_device_errors: no device error word");
  cudaStream_t s = gfe::as_stream(stream);
  unsigned v = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&v, w, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(unsigned), s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  *bits_host = v;
  return GFE_OK;
}

// ---------------------------------------------------------------------------------------------
// stage timing
// ---------------------------------------------------------------------------------------------
#include <utility>
#include <vector>

namespace {
bool g_profile = false;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_stage_events[GFE_STAGE_COUNT];
std::mutex g_prof_mu;
}  // namespace

namespace gfe {

bool profiling() { return g_profile; }

void* stage_begin(int stage, cudaStream_t s) {
  if (!g_profile || stage < 0 || stage >= GFE_STAGE_COUNT) return nullptr;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return nullptr;
  if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return nullptr; }
  cudaEventRecord(a, s);
  auto* pr = new std::pair<cudaEvent_t, cudaEvent_t>(a, b);
  return pr;
}

void stage_end(int stage, void* token, cudaStream_t s, int launches) {
  if (!token) return;
  auto* pr = static_cast<std::pair<cudaEvent_t, cudaEvent_t>*>(token);
  cudaEventRecord(pr->second, s);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (int i = 0; i < launches; ++i) {
    // one entry per launch keeps the launch count; only the first carries the events
    g_stage_events[stage].push_back(i == 0 ? *pr : std::make_pair(cudaEvent_t(nullptr), cudaEvent_t(nullptr)));
  }
  delete pr;
}

}  // namespace gfe

extern "C" int gfe_profile_enable(int on) {
  g_profile = on != 0;
  return GFE_OK;
}

extern "C" int gfe_profile_read(int stage, double* ms_host, int64_t* launches_host, int reset) {
  if (stage < 0 || stage >= GFE_STAGE_COUNT || !ms_host)
    return gfe::set_error(GFE_ERR_ARG, "gfe_profile_read: invalid stage %d", stage);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  double tot = 0.0;
  for (auto& pr : g_stage_events[stage]) {
    if (!pr.first) continue;
    if (cudaEventSynchronize(pr.second) != cudaSuccess)
      return gfe::set_error(GFE_ERR_CUDA, "gfe_profile_read: event wait failed");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pr.first, pr.second);
    tot += ms;
  }
  *ms_host = tot;
  if (launches_host) *launches_host = (int64_t)g_stage_events[stage].size();
  if (reset) {
    for (auto& pr : g_stage_events[stage])
      if (pr.first) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    g_stage_events[stage].clear();
  }
  return GFE_OK;
}

// ---------------------------------------------------------------------------------------------
// arithmetic-rate probe
// ---------------------------------------------------------------------------------------------
namespace {
template <typename T>
__global__ void fma_chain(T* out, int iters, T a, T b) {
  // 8 independent chains per thread keep the pipe full; each step is one FMA per chain
  T x0 = threadIdx.x * T(1e-7), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == T(-1.2345)) out[blockIdx.x] = s;  // keeps the chains alive
}
}  // namespace

extern "C" int gfe_probe_fma_rate(int32_t precision, double* gflops_host, void* stream) {
  if (!gflops_host) return gfe::set_error(GFE_ERR_ARG, "gfe_probe_fma_rate: null output");
  cudaStream_t s = gfe::as_stream(stream);
  const int blocks = gfe::sm_count() * 8, threads = 256;
  const int iters = precision == GFE_FP64 ? 4096 : 65536;
  void* out = nullptr;
  int rc = gfe::scratch_alloc(&out, sizeof(double) * blocks, s, "probe");
  if (rc) return rc;
  cudaEvent_t a, b;
  GFE_CUDA_TRY(cudaEventCreate(&a));
  GFE_CUDA_TRY(cudaEventCreate(&b));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, s);
    if (precision == GFE_FP64)
      fma_chain<double><<<blocks, threads, 0, s>>>((double*)out, iters, 0.999999, 1e-9);
    else
      fma_chain<float><<<blocks, threads, 0, s>>>((float*)out, iters, 0.999999f, 1e-9f);
    cudaEventRecord(b, s);
    GFE_CUDA_TRY(cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  gfe::scratch_free(out, s);
  GFE_LAUNCH_CHECK("gfe_probe_fma_rate");
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *gflops_host = flops / (best * 1e-3) / 1e9;
  return GFE_OK;
}
