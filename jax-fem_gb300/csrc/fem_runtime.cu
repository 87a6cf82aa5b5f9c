// Library runtime: error text, device queries, version.
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "fem_common.cuh"

namespace fem {

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

void note_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return FEM_OK;
}

int sm_count() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cache[dev] = n;
  }
  return cache[dev];
}

}  // namespace fem

extern "C" const char* fem_last_error(void) { return fem::g_last_error.c_str(); }

extern "C" int fem_version(void) { return 100; }

extern "C" uint64_t fem_kernel_launches(void) { return (uint64_t)fem::g_launches.load(); }
