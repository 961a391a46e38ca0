// refcuda_loader.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Loads oracle/_ref/refcuda.cubin (the reference's CUDA kernels, see
// refcuda.cu) into the calling thread's current CUDA context and launches its
// kernels by index with the reference's argument list (q, p, particle_number,
// dt, CL2, list, number_of_partners, pointer; cuda/kernel.cuh:5-13), the way
// the reference's measure() does (cuda/force_cuda.cu:319-342).  The CUDA
// driver library is opened at run time, so this library loads on machines
// without a GPU and fails only when used there.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <dlfcn.h>
#include <string>
#include <vector>

namespace {

typedef int CUresult;
typedef struct CUctx_st* CUcontext;
typedef struct CUmod_st* CUmodule;
typedef struct CUfunc_st* CUfunction;
typedef struct CUstream_st* CUstream;

struct Driver {
  void* h = nullptr;
  CUresult (*ctx_get_current)(CUcontext*) = nullptr;
  CUresult (*module_load_data)(CUmodule*, const void*) = nullptr;
  CUresult (*module_function_count)(unsigned*, CUmodule) = nullptr;
  CUresult (*module_enumerate)(CUfunction*, unsigned, CUmodule) = nullptr;
  CUresult (*func_name)(const char**, CUfunction) = nullptr;
  CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                     unsigned, CUstream, void**, void**) = nullptr;
  bool open() {
    if (h) return true;
    h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) return false;
    auto sym = [&](const char* n) { return dlsym(h, n); };
    ctx_get_current = (CUresult(*)(CUcontext*))sym("cuCtxGetCurrent");
    module_load_data = (CUresult(*)(CUmodule*, const void*))sym("cuModuleLoadData");
    module_function_count = (CUresult(*)(unsigned*, CUmodule))sym("cuModuleGetFunctionCount");
    module_enumerate =
        (CUresult(*)(CUfunction*, unsigned, CUmodule))sym("cuModuleEnumerateFunctions");
    func_name = (CUresult(*)(const char**, CUfunction))sym("cuFuncGetName");
    launch = (CUresult(*)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                          unsigned, CUstream, void**, void**))sym("cuLaunchKernel");
    return ctx_get_current && module_load_data && module_function_count && module_enumerate &&
           func_name && launch;
  }
};

Driver g_drv;
CUmodule g_mod = nullptr;
std::vector<CUfunction> g_funcs;
std::vector<std::string> g_names;

}  // namespace

extern "C" {

// Returns the number of kernels in the cubin, or a negative code: -1 driver
// library missing, -2 no current context, -3 file unreadable, -4 load failed.
int rc_load(const char* path) {
  if (!g_drv.open()) return -1;
  CUcontext ctx = nullptr;
  if (g_drv.ctx_get_current(&ctx) != 0 || !ctx) return -2;
  FILE* f = std::fopen(path, "rb");
  if (!f) return -3;
  std::vector<char> img;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) img.insert(img.end(), buf, buf + got);
  std::fclose(f);
  if (g_drv.module_load_data(&g_mod, img.data()) != 0) return -4;
  unsigned count = 0;
  if (g_drv.module_function_count(&count, g_mod) != 0) return -4;
  g_funcs.assign(count, nullptr);
  if (count && g_drv.module_enumerate(g_funcs.data(), count, g_mod) != 0) return -4;
  g_names.clear();
  for (CUfunction fn : g_funcs) {
    const char* name = nullptr;
    g_names.emplace_back(g_drv.func_name(&name, fn) == 0 && name ? name : "");
  }
  return (int)count;
}

// Mangled name of kernel k ("" when out of range).
const char* rc_name(int k) {
  return k >= 0 && k < (int)g_names.size() ? g_names[(size_t)k].c_str() : "";
}

// One launch of kernel k: grid x block threads on `stream` (NULL: legacy).
int rc_launch(int k, int grid, int block, const void* q, void* p, int32_t n, double dt,
              double cl2, const int32_t* list, const int32_t* np, const int32_t* ptr,
              void* stream) {
  if (k < 0 || k >= (int)g_funcs.size() || grid < 1 || block < 1) return -1;
  void* args[] = {&q, &p, &n, &dt, &cl2, &list, &np, &ptr};
  return g_drv.launch(g_funcs[(size_t)k], (unsigned)grid, 1, 1, (unsigned)block, 1, 1, 0,
                      (CUstream)stream, args, nullptr);
}

}  // extern "C"
