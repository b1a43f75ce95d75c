// jit.cpp — NVRTC compilation of field-function modules for sm_103a.
//
// Replaces the shader-module creation of the reference
// (device.create_shader_module + create_compute_pipeline,
// src/main_view.rs:662-673): the generated CUDA C plus the embedded march
// kernels are compiled to a cubin and loaded with the runtime's library API
// (no driver-API link, so the shared library loads on machines without a
// GPU).  Compiled cubins are cached per (source, options, headers) in memory
// and, when LINON_CACHE_DIR is set, on disk.
#include <nvrtc.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "internal.hpp"

namespace linon {
namespace {

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t headers_hash() {
  static uint64_t h = [] {
    uint64_t x = 1469598103934665603ull;
    for (int i = 0; i < kEmbeddedDeviceSourceCount; ++i) {
      x = fnv1a(kEmbeddedDeviceSources[i].name, x);
      x = fnv1a(kEmbeddedDeviceSources[i].text, x);
    }
    return x;
  }();
  return h;
}

std::mutex g_mu;
std::map<std::string, std::vector<char>> g_cubins;              // key -> cubin
std::map<std::string, std::shared_ptr<JitModule>> g_modules;    // key -> loaded module (device 0..n)

std::vector<std::string> options(bool precise) {
  std::vector<std::string> o = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo",
                                "--device-as-default-execution-space"};
  if (precise) {
    o.push_back("--fmad=false");
    o.push_back("-DLINON_PRECISE=1");
  } else {
    // fast modules: the hardware reciprocal / square-root sequences (about
    // 1 ulp) instead of the correctly rounded ones
    o.push_back("--prec-div=false");
    o.push_back("--prec-sqrt=false");
  }
  if (std::getenv("LINON_JIT_VERBOSE")) o.push_back("--ptxas-options=--verbose");
  // extra NVRTC options (space separated), e.g. "-maxrregcount=64" or
  // "-DLINON_SINCOS_POLY" (see wgsl_rt.cuh); they are part of the cache key
  if (const char* extra = std::getenv("LINON_JIT_OPTIONS")) {
    std::istringstream is(extra);
    std::string opt;
    while (is >> opt) o.push_back(opt);
  }
  return o;
}

bool read_file(const std::string& path, std::vector<char>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return !out.empty();
}

void write_file(const std::string& path, const std::vector<char>& data) {
  std::string tmp = path + ".tmp" + std::to_string(::getpid());
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return;
    f.write(data.data(), std::streamsize(data.size()));
  }
  std::rename(tmp.c_str(), path.c_str());
}

int nvrtc_compile(const std::string& source, const std::vector<std::string>& opts,
                  std::vector<char>& cubin, std::string& log) {
  std::vector<const char*> hdr_text, hdr_name;
  for (int i = 0; i < kEmbeddedDeviceSourceCount; ++i) {
    hdr_text.push_back(kEmbeddedDeviceSources[i].text);
    hdr_name.push_back(kEmbeddedDeviceSources[i].name);
  }
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, source.c_str(), "linon_field_module.cu",
                                     int(hdr_text.size()), hdr_text.data(), hdr_name.data());
  if (r != NVRTC_SUCCESS) {
    log = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r);
    return LINON_ECOMPILE;
  }
  std::vector<const char*> o;
  for (auto& s : opts) o.push_back(s.c_str());
  r = nvrtcCompileProgram(prog, int(o.size()), o.data());
  size_t log_size = 0;
  nvrtcGetProgramLogSize(prog, &log_size);
  if (log_size > 1) {
    std::string l(log_size, '\0');
    nvrtcGetProgramLog(prog, &l[0]);
    while (!l.empty() && l.back() == '\0') l.pop_back();
    log = l;
  }
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    log = std::string("NVRTC compilation failed (") + nvrtcGetErrorString(r) + "):\n" + log;
    return LINON_ECOMPILE;
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin.resize(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  if (n == 0) {
    log = "NVRTC produced no cubin";
    return LINON_ECOMPILE;
  }
  return LINON_OK;
}

}  // namespace

int jit_check(const std::string& source, bool precise, std::string& log, size_t* cubin_bytes) {
  std::vector<std::string> opts = options(precise);
  opts.push_back("--ptxas-options=--verbose");
  std::vector<char> cubin;
  int st = nvrtc_compile(source, opts, cubin, log);
  if (cubin_bytes) *cubin_bytes = cubin.size();
  return st;
}

int jit_compile(const std::string& source, bool precise, const std::vector<std::string>& kernel_names,
                std::shared_ptr<JitModule>& out, std::string& log) {
  const std::vector<std::string> opts = options(precise);
  std::string optstr;
  for (auto& s : opts) optstr += s + " ";
  int major = 0, minor = 0;
  nvrtcVersion(&major, &minor);
  char keybuf[64];
  uint64_t h = fnv1a(source, headers_hash());
  h = fnv1a(optstr, h);
  h = fnv1a(std::to_string(major) + "." + std::to_string(minor), h);
  std::snprintf(keybuf, sizeof keybuf, "%016llx", (unsigned long long)h);
  const std::string key = keybuf;
  int dev = 0;
  cudaGetDevice(&dev);
  const std::string mkey = key + "@" + std::to_string(dev);

  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_modules.find(mkey);
  if (it != g_modules.end()) {
    out = it->second;
    return LINON_OK;
  }
  auto t0 = std::chrono::steady_clock::now();
  std::vector<char>& cubin = g_cubins[key];
  if (cubin.empty()) {
    const char* dir = std::getenv("LINON_CACHE_DIR");
    std::string path = dir ? std::string(dir) + "/linon_" + key + ".cubin" : std::string();
    if (path.empty() || !read_file(path, cubin)) {
      int st = nvrtc_compile(source, opts, cubin, log);
      if (st != LINON_OK) {
        g_cubins.erase(key);
        return st;
      }
      if (!path.empty()) write_file(path, cubin);
    }
  }
  auto mod = std::make_shared<JitModule>();
  mod->key = key;
  cudaError_t e = cudaLibraryLoadData(&mod->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) return cuda_error(e, "cudaLibraryLoadData");
  for (const auto& name : kernel_names) {
    cudaKernel_t k;
    e = cudaLibraryGetKernel(&k, mod->lib, name.c_str());
    if (e != cudaSuccess) return cuda_error(e, ("cudaLibraryGetKernel " + name).c_str());
    mod->kernels[name] = k;
  }
  mod->compile_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  g_modules[mkey] = mod;
  out = mod;
  return LINON_OK;
}

}  // namespace linon
