// Run-time compiled kernels: the user weak-form kernels of the Problem API
// (get_universal_kernel, get_universal_kernels_surface).  The Python layer traces the user's
// function into CUDA C++ source (jax-fem_gb300/jit.py); this file compiles that source with NVRTC
// for the current device, loads it, and launches its cell / face kernels with one fixed parameter
// block (fem_jit_params_t).  NVRTC is opened at run time (libnvrtc.so.13), the driver entry points
// come from the runtime (cudaGetDriverEntryPointByVersion), so the library links neither.
#include <cuda.h>
#include <dlfcn.h>

#include <functional>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "fem_common.cuh"

namespace fem {
namespace {

typedef int (*nvrtcCreateProgram_t)(void**, const char*, const char*, int, const char* const*, const char* const*);
typedef int (*nvrtcCompileProgram_t)(void*, int, const char* const*);
typedef int (*nvrtcGetSize_t)(void*, size_t*);
typedef int (*nvrtcGetData_t)(void*, char*);
typedef int (*nvrtcDestroyProgram_t)(void**);
typedef const char* (*nvrtcGetErrorString_t)(int);

struct Nvrtc {
  bool ok = false;
  std::string why;
  nvrtcCreateProgram_t create = nullptr;
  nvrtcCompileProgram_t compile = nullptr;
  nvrtcGetSize_t log_size = nullptr, cubin_size = nullptr;
  nvrtcGetData_t log = nullptr, cubin = nullptr;
  nvrtcDestroyProgram_t destroy = nullptr;
  nvrtcGetErrorString_t err = nullptr;
};

Nvrtc& nvrtc() {
  static Nvrtc N;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = nullptr;
    for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"}) {
      h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) {
      N.why = "NVRTC (libnvrtc.so.13) could not be opened: " + std::string(dlerror() ? dlerror() : "not found");
      return;
    }
    N.create = (nvrtcCreateProgram_t)dlsym(h, "nvrtcCreateProgram");
    N.compile = (nvrtcCompileProgram_t)dlsym(h, "nvrtcCompileProgram");
    N.log_size = (nvrtcGetSize_t)dlsym(h, "nvrtcGetProgramLogSize");
    N.log = (nvrtcGetData_t)dlsym(h, "nvrtcGetProgramLog");
    N.cubin_size = (nvrtcGetSize_t)dlsym(h, "nvrtcGetCUBINSize");
    N.cubin = (nvrtcGetData_t)dlsym(h, "nvrtcGetCUBIN");
    N.destroy = (nvrtcDestroyProgram_t)dlsym(h, "nvrtcDestroyProgram");
    N.err = (nvrtcGetErrorString_t)dlsym(h, "nvrtcGetErrorString");
    N.ok = N.create && N.compile && N.log_size && N.log && N.cubin_size && N.cubin && N.destroy && N.err;
    if (!N.ok) N.why = "NVRTC library lacks an expected entry point";
  });
  return N;
}

typedef CUresult (*cuModuleLoadData_t)(CUmodule*, const void*);
typedef CUresult (*cuModuleGetFunction_t)(CUfunction*, CUmodule, const char*);
typedef CUresult (*cuLaunchKernel_t)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                                     CUstream, void**, void**);

struct Driver {
  bool ok = false;
  std::string why;
  cuModuleLoadData_t load = nullptr;
  cuModuleGetFunction_t get = nullptr;
  cuLaunchKernel_t launch = nullptr;
};

Driver& driver() {
  static Driver D;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    auto sym = [&](const char* name) -> void* {
      p = nullptr;
      if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
          q != cudaDriverEntryPointSuccess)
        return nullptr;
      return p;
    };
    D.load = (cuModuleLoadData_t)sym("cuModuleLoadData");
    D.get = (cuModuleGetFunction_t)sym("cuModuleGetFunction");
    D.launch = (cuLaunchKernel_t)sym("cuLaunchKernel");
    D.ok = D.load && D.get && D.launch;
    if (!D.ok) D.why = "CUDA driver entry points for module loading are unavailable";
  });
  return D;
}

struct Module {
  CUmodule mod = nullptr;
  std::unordered_map<std::string, CUfunction> fns;
};

std::mutex g_mu;
std::vector<Module> g_mods;                                  // handle = index + 1
std::unordered_map<std::string, size_t> g_by_source;         // (device, source) -> index

}  // namespace
}  // namespace fem

extern "C" int fem_jit_load(const char* source, void** module) {
  using namespace fem;
  FEM_REQUIRE(source && module, "NULL argument");
  Nvrtc& N = nvrtc();
  if (!N.ok) return fail(FEM_ERR_UNSUPPORTED, N.why);
  Driver& D = driver();
  if (!D.ok) return fail(FEM_ERR_UNSUPPORTED, D.why);
  int dev = 0, major = 0, minor = 0;
  FEM_CUDA(cudaGetDevice(&dev));
  FEM_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  FEM_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  FEM_CUDA(cudaFree(nullptr));   // make the runtime's primary context current for the driver calls
  const std::string key = std::to_string(dev) + "\n" + source;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_by_source.find(key);
    if (it != g_by_source.end()) {
      *module = reinterpret_cast<void*>(it->second + 1);
      return FEM_OK;
    }
  }
  void* prog = nullptr;
  int r = N.create(&prog, source, "fem_jit.cu", 0, nullptr, nullptr);
  if (r) return fail(FEM_ERR_UNSUPPORTED, std::string("nvrtcCreateProgram: ") + N.err(r));
  const std::string arch = "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) +
                           (major >= 9 ? "a" : "");
  const char* opts[] = {arch.c_str(), "--std=c++17", "--fmad=true", "-default-device"};
  r = N.compile(prog, 4, opts);
  if (r) {
    size_t n = 0;
    N.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) N.log(prog, &log[0]);
    N.destroy(&prog);
    return fail(FEM_ERR_ARG, std::string("NVRTC compilation of a generated kernel failed: ") + N.err(r) + "\n" + log);
  }
  size_t n = 0;
  N.cubin_size(prog, &n);
  std::vector<char> cubin(n);
  N.cubin(prog, cubin.data());
  N.destroy(&prog);
  CUmodule mod = nullptr;
  const CUresult cr = D.load(&mod, cubin.data());
  if (cr != CUDA_SUCCESS) return fail(FEM_ERR_CUDA, "cuModuleLoadData failed: " + std::to_string((int)cr));
  std::lock_guard<std::mutex> lk(g_mu);
  g_mods.push_back(Module{mod, {}});
  g_by_source[key] = g_mods.size() - 1;
  *module = reinterpret_cast<void*>(g_mods.size());
  return FEM_OK;
}

extern "C" int fem_jit_launch(void* module, const char* kernel, const fem_jit_params_t* params, int64_t n_items,
                              void* stream) {
  using namespace fem;
  FEM_REQUIRE(module && kernel && params, "NULL argument");
  FEM_REQUIRE(n_items >= 0, "n_items < 0");
  if (n_items == 0) return FEM_OK;
  Driver& D = driver();
  if (!D.ok) return fail(FEM_ERR_UNSUPPORTED, D.why);
  CUfunction fn = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t idx = reinterpret_cast<size_t>(module);
    FEM_REQUIRE(idx >= 1 && idx <= g_mods.size(), "unknown JIT module handle");
    Module& M = g_mods[idx - 1];
    auto it = M.fns.find(kernel);
    if (it == M.fns.end()) {
      const CUresult cr = D.get(&fn, M.mod, kernel);
      if (cr != CUDA_SUCCESS) return fail(FEM_ERR_ARG, std::string("generated kernel not found: ") + kernel);
      M.fns[kernel] = fn;
    } else {
      fn = it->second;
    }
  }
  constexpr unsigned threads = 128;
  int64_t blocks = (n_items + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  fem_jit_params_t P = *params;
  void* args[] = {&P};
  const CUresult cr = D.launch(fn, (unsigned)blocks, 1, 1, threads, 1, 1, 0, (CUstream)as_stream(stream), args,
                               nullptr);
  if (cr != CUDA_SUCCESS) return fail(FEM_ERR_CUDA, "cuLaunchKernel failed: " + std::to_string((int)cr));
  note_launches(1);
  return check_launch(kernel);
}
