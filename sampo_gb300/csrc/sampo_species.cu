// sampo_species.cu - user species headers compiled at run time.
//
// The reference compiles its OpenCL kernels at start-up with the species
// header named on its command line (src/abms.c:565-568, lib_icl's
// runtime build, src/lib_icl.c:607-636). Here the step kernels
// (sampo_step_kernels.cuh and the headers it includes, embedded in the
// library as text by the build) are compiled by NVRTC with
// SAMPO_USER_SPECIES and the user's header, loaded through the CUDA driver
// API and launched by the same launchers as the built-in kernels
// (KParams::ks). NVRTC is opened with dlopen, the driver entry points come
// from the CUDA runtime, so the library needs neither at load time.
#include <cuda.h>
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "sampo_kernels.cuh"

// the kernel sources, embedded by the build (sampo_jit_sources.cpp)
extern "C" const char* const sampo_jit_names[];
extern "C" const char* const sampo_jit_texts[];
extern "C" const int sampo_jit_count;

using namespace sampo;

namespace {

// ---- NVRTC, opened on first use ----
struct Nvrtc {
  bool ok = false;
  std::string why;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcAddNameExpression) add_name = nullptr;
  decltype(&nvrtcGetLoweredName) lowered = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

void open_nvrtc(Nvrtc& n);

const Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] { open_nvrtc(n); });
  return n;
}

void open_nvrtc(Nvrtc& n) {
  const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  void* h = nullptr;
  for (const char* nm : names)
    if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
  if (!h) {
    n.why = "NVRTC (libnvrtc.so) not found";
    return;
  }
#define SAMPO_SYM(field, sym) n.field = reinterpret_cast<decltype(n.field)>(dlsym(h, #sym))
  SAMPO_SYM(create, nvrtcCreateProgram);
  SAMPO_SYM(compile, nvrtcCompileProgram);
  SAMPO_SYM(add_name, nvrtcAddNameExpression);
  SAMPO_SYM(lowered, nvrtcGetLoweredName);
  SAMPO_SYM(cubin_size, nvrtcGetCUBINSize);
  SAMPO_SYM(cubin, nvrtcGetCUBIN);
  SAMPO_SYM(log_size, nvrtcGetProgramLogSize);
  SAMPO_SYM(log, nvrtcGetProgramLog);
  SAMPO_SYM(destroy, nvrtcDestroyProgram);
#undef SAMPO_SYM
  n.ok = n.create && n.compile && n.add_name && n.lowered && n.cubin_size && n.cubin && n.log_size && n.log && n.destroy;
  if (!n.ok) n.why = "NVRTC lacks an entry point this library needs";
  return;
}

// ---- driver API entry points, from the runtime ----
struct Driver;
void open_driver(Driver& d);
struct Driver {
  bool ok = false;
  CUresult (*module_load)(CUmodule*, const void*) = nullptr;
  CUresult (*module_unload)(CUmodule) = nullptr;
  CUresult (*get_function)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream, void**,
                     void**) = nullptr;
  CUresult (*set_attr)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
};

const Driver& driver() {
  static Driver d;
  static std::once_flag once;
  std::call_once(once, [] { open_driver(d); });
  return d;
}

void open_driver(Driver& d) {
  auto get = [](const char* sym, void** fp) {
    cudaDriverEntryPointQueryResult q;
    return cudaGetDriverEntryPointByVersion(sym, fp, 12000, cudaEnableDefault, &q) == cudaSuccess &&
           q == cudaDriverEntryPointSuccess && *fp;
  };
  d.ok = get("cuModuleLoadData", (void**)&d.module_load) && get("cuModuleUnload", (void**)&d.module_unload) &&
         get("cuModuleGetFunction", (void**)&d.get_function) && get("cuLaunchKernel", (void**)&d.launch) &&
         get("cuFuncSetAttribute", (void**)&d.set_attr) &&
         get("cuOccupancyMaxActiveBlocksPerMultiprocessor", (void**)&d.occupancy);
}

// the kernels of one compiled species, in KID_* order
const char* const kKernelNames[KID_N] = {"&sampo::k_count<4>",   "&sampo::k_scatter<4>", "&sampo::k_publish",
                                         "&sampo::k_init_eggs",  "&sampo::k_pool_stats", "&sampo::k_histogram",
                                         "&sampo::k_trial_reset"};

// standard headers the kernel sources include, reduced to what NVRTC lacks,
// and the reference's headers a species header includes (the prelude defines
// their contents)
const char* const kStubNames[] = {"stdint.h", "stddef.h", "string.h", "device_types.h", "agent.h", "gpuRand.h"};
const char* const kStubTexts[] = {
    "#pragma once\ntypedef signed char int8_t; typedef unsigned char uint8_t; typedef short int16_t;\n"
    "typedef unsigned short uint16_t; typedef int int32_t; typedef unsigned int uint32_t;\n"
    "typedef long long int64_t; typedef unsigned long long uint64_t;\n",
    "#pragma once\n", "#pragma once\n", "#pragma once\n", "#pragma once\n", "#pragma once\n"};

}  // namespace

struct sampo_species {
  int device = 0;
  CUmodule module = nullptr;
  CUfunction fn[KID_N] = {};
  std::string log;
};

namespace sampo {

cudaError_t species_launch(const void* ks, int kid, dim3 grid, dim3 block, size_t smem, cudaStream_t st, void** args) {
  const sampo_species* sp = static_cast<const sampo_species*>(ks);
  const CUresult r = driver().launch(sp->fn[kid], grid.x, grid.y, grid.z, block.x, block.y, block.z, (unsigned)smem,
                                     (CUstream)st, args, nullptr);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorLaunchFailure;
}

int species_occupancy(const void* ks, int kid, int threads, size_t smem) {
  const sampo_species* sp = static_cast<const sampo_species*>(ks);
  int per = 0;
  if (driver().occupancy(&per, sp->fn[kid], threads, smem) != CUDA_SUCCESS) return 0;
  return per;
}

}  // namespace sampo

static void put_log(char* buf, size_t size, const std::string& s) {
  if (!buf || !size) return;
  const size_t n = s.size() < size - 1 ? s.size() : size - 1;
  memcpy(buf, s.data(), n);
  buf[n] = 0;
}

// Compiles the step kernels against the header text for sm_<sm>a; on
// success *cubin holds the code and *prog the program (for the lowered names).
static int compile_kernels(const char* name, const char* text, int sm, std::string& clog, std::vector<char>& cubin,
                           nvrtcProgram* prog_out) {
  const Nvrtc& rt = nvrtc();
  if (!rt.ok) {
    clog = rt.why;
    return SAMPO_ERR_UNSUPPORTED;
  }
  // headers: the embedded kernel sources, the stubs, and the user's header
  std::vector<const char*> hnames, htexts;
  for (int i = 0; i < sampo_jit_count; i++) {
    hnames.push_back(sampo_jit_names[i]);
    htexts.push_back(sampo_jit_texts[i]);
  }
  for (size_t i = 0; i < sizeof(kStubNames) / sizeof(kStubNames[0]); i++) {
    hnames.push_back(kStubNames[i]);
    htexts.push_back(kStubTexts[i]);
  }
  hnames.push_back("sampo_user_species.h");
  htexts.push_back(text);
  const char* src = "#include \"sampo_step_kernels.cuh\"\n";
  nvrtcProgram prog = nullptr;
  if (rt.create(&prog, src, name ? name : "species.cu", (int)hnames.size(), htexts.data(), hnames.data()) != NVRTC_SUCCESS) {
    clog = "nvrtcCreateProgram failed";
    return SAMPO_ERR_INTERNAL;
  }
  for (const char* k : kKernelNames) rt.add_name(prog, k);
  const std::string arch = "-arch=sm_" + std::to_string(sm) + "a";
  const char* opts[] = {arch.c_str(), "-default-device", "-std=c++17", "--fmad=false", "-prec-div=true",
                        "-prec-sqrt=true", "-DSAMPO_USER_SPECIES=1"};
  const nvrtcResult cr = rt.compile(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
  size_t ls = 0;
  rt.log_size(prog, &ls);
  clog.assign(ls, '\0');
  if (ls) rt.log(prog, &clog[0]);
  while (!clog.empty() && clog.back() == '\0') clog.pop_back();
  if (cr != NVRTC_SUCCESS) {
    rt.destroy(&prog);
    return SAMPO_ERR_SPECIES;
  }
  size_t cs = 0;
  rt.cubin_size(prog, &cs);
  cubin.resize(cs);
  rt.cubin(prog, cubin.data());
  if (prog_out) *prog_out = prog;
  else rt.destroy(&prog);
  return SAMPO_OK;
}

extern "C" int sampo_species_check_text(const char* name, const char* text, int sm, char* log, size_t log_size) {
  if (!text || sm <= 0) return SAMPO_ERR_ARG;
  std::string clog;
  std::vector<char> cubin;
  const int rc = compile_kernels(name, text, sm, clog, cubin, nullptr);
  put_log(log, log_size, clog);
  return rc;
}

extern "C" int sampo_species_compile_text(const char* name, const char* text, int device, char* log, size_t log_size,
                                          sampo_species** out) {
  if (!text || !out) return SAMPO_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess || cudaFree(nullptr) != cudaSuccess) {
    put_log(log, log_size, "no CUDA device");
    return SAMPO_ERR_CUDA;
  }
  const Driver& drv = driver();
  if (!drv.ok) {
    put_log(log, log_size, "CUDA driver entry points unavailable");
    return SAMPO_ERR_UNSUPPORTED;
  }
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  std::string clog;
  std::vector<char> cubin;
  nvrtcProgram prog = nullptr;
  const int rc = compile_kernels(name, text, major * 10 + minor, clog, cubin, &prog);
  if (rc != SAMPO_OK) {
    put_log(log, log_size, clog);
    return rc;
  }
  const Nvrtc& rt = nvrtc();
  sampo_species* sp = new sampo_species();
  sp->device = device;
  sp->log = clog;
  CUresult r = drv.module_load(&sp->module, cubin.data());
  for (int k = 0; k < KID_N && r == CUDA_SUCCESS; k++) {
    const char* lowered = nullptr;
    if (rt.lowered(prog, kKernelNames[k], &lowered) != NVRTC_SUCCESS || !lowered) {
      r = CUDA_ERROR_NOT_FOUND;
      break;
    }
    r = drv.get_function(&sp->fn[k], sp->module, lowered);
  }
  rt.destroy(&prog);
  if (r == CUDA_SUCCESS) r = drv.set_attr(sp->fn[KID_COUNT], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)count_smem_max());
  if (r == CUDA_SUCCESS)
    r = drv.set_attr(sp->fn[KID_SCATTER], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)scatter_smem_max());
  if (r != CUDA_SUCCESS) {
    if (sp->module) drv.module_unload(sp->module);
    delete sp;
    put_log(log, log_size, "loading the compiled kernels failed (CUresult " + std::to_string((int)r) + ")");
    return SAMPO_ERR_CUDA;
  }
  put_log(log, log_size, clog);
  *out = sp;
  return SAMPO_OK;
}

extern "C" int sampo_species_compile(const char* header_path, int device, char* log, size_t log_size, sampo_species** out) {
  if (!header_path || !out) return SAMPO_ERR_ARG;
  FILE* f = fopen(header_path, "rb");
  if (!f) {
    put_log(log, log_size, std::string("cannot open ") + header_path);
    return SAMPO_ERR_IO;
  }
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  fclose(f);
  return sampo_species_compile_text(header_path, text.c_str(), device, log, log_size, out);
}

extern "C" int sampo_species_device(const sampo_species* sp) { return sp ? sp->device : -1; }

extern "C" void sampo_species_free(sampo_species* sp) {
  if (!sp) return;
  if (sp->module && driver().ok) {
    cudaSetDevice(sp->device);
    driver().module_unload(sp->module);
  }
  delete sp;
}
