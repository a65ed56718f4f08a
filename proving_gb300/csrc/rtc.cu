// Run-time compiled constraint kernels: the generic path of the constraint
// framework. proving_gb300/framework.py turns an AIR's constraints, written
// against an evaluator like the reference's ExprEvaluator
// (crates/constraint-framework/src/expr/evaluator.rs:58-123), into the source of
// one kernel with a fixed signature; this file compiles it with NVRTC for
// sm_103a, loads the cubin through the runtime's library API, and launches it
// over an evaluation domain like the hand-written composition kernels
// (evaluate_constraint_quotients_on_domain,
// crates/constraint-framework/src/prover/component_prover.rs:111-193).
//
// NVRTC is opened at run time (dlopen), so the library loads where it is absent
// and only the compile entry point reports it missing.
#include <dlfcn.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "field.cuh"

namespace cs {
namespace {

// The NVRTC entry points used here (nvrtc.h, CUDA 13).
typedef struct _nvrtcProgram* nvrtcProgram;
typedef int nvrtcResult;  // 0 = NVRTC_SUCCESS
struct Nvrtc {
  nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*);
  nvrtcResult (*compile)(nvrtcProgram, int, const char* const*);
  nvrtcResult (*log_size)(nvrtcProgram, size_t*);
  nvrtcResult (*log)(nvrtcProgram, char*);
  nvrtcResult (*cubin_size)(nvrtcProgram, size_t*);
  nvrtcResult (*cubin)(nvrtcProgram, char*);
  nvrtcResult (*destroy)(nvrtcProgram*);
  bool ok = false;
  std::string why;
};

Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    std::vector<std::string> names;
    if (const char* home = std::getenv("CUDA_HOME")) names.push_back(std::string(home) + "/lib64/libnvrtc.so.13");
    names.push_back("libnvrtc.so.13");
    names.push_back("libnvrtc.so");
    names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    void* h = nullptr;
    for (const std::string& name : names)
      if ((h = dlopen(name.c_str(), RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
    if (h == nullptr) {
      n.why = "libnvrtc.so.13 not found";
      return;
    }
    n.create = reinterpret_cast<decltype(n.create)>(dlsym(h, "nvrtcCreateProgram"));
    n.compile = reinterpret_cast<decltype(n.compile)>(dlsym(h, "nvrtcCompileProgram"));
    n.log_size = reinterpret_cast<decltype(n.log_size)>(dlsym(h, "nvrtcGetProgramLogSize"));
    n.log = reinterpret_cast<decltype(n.log)>(dlsym(h, "nvrtcGetProgramLog"));
    n.cubin_size = reinterpret_cast<decltype(n.cubin_size)>(dlsym(h, "nvrtcGetCUBINSize"));
    n.cubin = reinterpret_cast<decltype(n.cubin)>(dlsym(h, "nvrtcGetCUBIN"));
    n.destroy = reinterpret_cast<decltype(n.destroy)>(dlsym(h, "nvrtcDestroyProgram"));
    n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
    if (!n.ok) n.why = "libnvrtc lacks an entry point";
  });
  return n;
}

struct RtcKernel {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t fn = nullptr;
  cudaKernel_t fn_frac = nullptr;  // cs_air_fractions, for an AIR with LogUp batches
  uint32_t n_cols = 0, n_constraints = 0, n_params = 0, n_frac_cols = 0, n_batches = 0;
};

cpoint rtc_point_at(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_rtc_available(void) {
  Nvrtc& n = nvrtc();
  CS_CHECK_ARG(n.ok, "rtc: %s", n.why.c_str());
  return CS_OK;
}

extern "C" cs_status cs_rtc_compile_air(const char* source, uint32_t n_headers, const char* const* header_sources,
                                        const char* const* header_names, uint32_t n_cols, uint32_t n_constraints,
                                        uint32_t n_params, void** handle_out, char* log_out, size_t log_capacity) {
  return cs_rtc_compile_air_logup(source, n_headers, header_sources, header_names, n_cols, n_constraints, n_params, 0,
                                  0, handle_out, log_out, log_capacity);
}

extern "C" cs_status cs_rtc_compile_air_logup(const char* source, uint32_t n_headers,
                                              const char* const* header_sources, const char* const* header_names,
                                              uint32_t n_cols, uint32_t n_constraints, uint32_t n_params,
                                              uint32_t n_frac_cols, uint32_t n_batches, void** handle_out,
                                              char* log_out, size_t log_capacity) {
  CS_CHECK_ARG(source != nullptr && handle_out != nullptr, "rtc_compile_air: null pointer");
  CS_CHECK_ARG(n_batches <= 1024 && (n_batches > 0 || n_frac_cols == 0), "rtc_compile_air: %u LogUp batches",
               n_batches);
  CS_CHECK_ARG(n_headers == 0 || (header_sources != nullptr && header_names != nullptr),
               "rtc_compile_air: null header table");
  Nvrtc& n = nvrtc();
  CS_CHECK_ARG(n.ok, "rtc_compile_air: %s", n.why.c_str());
  *handle_out = nullptr;
  nvrtcProgram prog = nullptr;
  if (n.create(&prog, source, "air.cu", (int)n_headers, header_sources, header_names) != 0) {
    set_error("rtc_compile_air: nvrtcCreateProgram failed");
    return CS_ERR_DEVICE;
  }
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17"};
  const nvrtcResult rc = n.compile(prog, 2, opts);
  size_t log_size = 0;
  n.log_size(prog, &log_size);
  std::string log(log_size, '\0');
  if (log_size > 0) n.log(prog, &log[0]);
  if (log_out != nullptr && log_capacity > 0) {
    const size_t k = std::min(log_capacity - 1, log.size());
    std::copy(log.begin(), log.begin() + k, log_out);
    log_out[k] = '\0';
  }
  if (rc != 0) {
    n.destroy(&prog);
    set_error("rtc_compile_air: compilation failed: %.400s", log.c_str());
    return CS_ERR_INVALID_ARG;
  }
  size_t cubin_size = 0;
  n.cubin_size(prog, &cubin_size);
  std::vector<char> cubin(cubin_size);
  n.cubin(prog, cubin.data());
  n.destroy(&prog);
  RtcKernel* k = new RtcKernel;
  cudaError_t e = cudaLibraryLoadData(&k->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&k->fn, k->lib, "cs_air_composition");
  if (e == cudaSuccess && n_batches > 0) e = cudaLibraryGetKernel(&k->fn_frac, k->lib, "cs_air_fractions");
  if (e != cudaSuccess) {
    if (k->lib != nullptr) cudaLibraryUnload(k->lib);
    delete k;
    return from_cuda(e, "rtc_compile_air: load");
  }
  k->n_cols = n_cols;
  k->n_constraints = n_constraints;
  k->n_params = n_params;
  k->n_frac_cols = n_frac_cols;
  k->n_batches = n_batches;
  *handle_out = k;
  return CS_OK;
}

extern "C" cs_status cs_rtc_air_fractions(void* handle, const uint32_t* const* h_cols, const uint32_t* h_params,
                                          uint32_t log_n, uint32_t* const* h_out, cs_stream stream) {
  CS_CHECK_ARG(handle != nullptr && h_out != nullptr, "rtc_air_fractions: null pointer");
  const RtcKernel* k = static_cast<const RtcKernel*>(handle);
  CS_CHECK_ARG(k->fn_frac != nullptr, "rtc_air_fractions: the AIR has no LogUp batches");
  CS_CHECK_ARG(k->n_frac_cols == 0 || h_cols != nullptr, "rtc_air_fractions: null column table");
  CS_CHECK_ARG(k->n_params == 0 || h_params != nullptr, "rtc_air_fractions: null parameters");
  CS_CHECK_ARG(log_n >= 1 && log_n <= 30, "rtc_air_fractions: log size %u", log_n);
  for (uint32_t c = 0; c < k->n_frac_cols; c++)
    CS_CHECK_ARG(h_cols[c] != nullptr, "rtc_air_fractions: column %u is null", c);
  for (uint32_t c = 0; c < 8 * k->n_batches; c++)
    CS_CHECK_ARG(h_out[c] != nullptr, "rtc_air_fractions: output %u is null", c);
  // one staging buffer: column pointers, output pointers, then the parameters
  const size_t n_words = 2 * (size_t)k->n_frac_cols + 16 * (size_t)k->n_batches + 4 * (size_t)k->n_params + 4;
  std::vector<uint32_t> host(n_words, 0);
  uint32_t* w = host.data();
  const auto put_ptr = [&](const void* p) {
    const uint64_t v = reinterpret_cast<uint64_t>(p);
    *w++ = (uint32_t)v;
    *w++ = (uint32_t)(v >> 32);
  };
  for (uint32_t c = 0; c < k->n_frac_cols; c++) put_ptr(h_cols[c]);
  for (uint32_t c = 0; c < 8 * k->n_batches; c++) put_ptr(h_out[c]);
  for (size_t i = 0; i < 4 * (size_t)k->n_params; i++) *w++ = h_params[i] % P;
  cudaStream_t st = to_stream(stream);
  uint32_t* dev = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&dev), sizeof(uint32_t) * n_words, st));
  cs_status result = CS_OK;
  cudaError_t e = cudaMemcpyAsync(dev, host.data(), sizeof(uint32_t) * n_words, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const uint32_t* const* cols = reinterpret_cast<const uint32_t* const*>(dev);
    uint32_t* const* out = reinterpret_cast<uint32_t* const*>(dev + 2 * k->n_frac_cols);
    const uint32_t* params = dev + 2 * (size_t)k->n_frac_cols + 16 * (size_t)k->n_batches;
    void* args[] = {&cols, &params, &log_n, &out};
    const uint32_t n = 1u << log_n;
    const uint32_t blocks = std::max(1u, std::min((n + 255) / 256, 152u * 8));
    e = cudaLaunchKernel(reinterpret_cast<const void*>(k->fn_frac), dim3(blocks), dim3(256), args, 0, st);
    note_launch();
  }
  if (e != cudaSuccess) result = from_cuda(e, "rtc_air_fractions");
  const cudaError_t ef = cudaFreeAsync(dev, st);
  if (result == CS_OK && ef != cudaSuccess) return from_cuda(ef, "cudaFreeAsync");
  return result;
}

extern "C" cs_status cs_rtc_kernel_shape(void* handle, uint32_t* n_cols, uint32_t* n_constraints, uint32_t* n_params) {
  CS_CHECK_ARG(handle != nullptr && n_cols != nullptr && n_constraints != nullptr && n_params != nullptr,
               "rtc_kernel_shape: null pointer");
  const RtcKernel* k = static_cast<const RtcKernel*>(handle);
  *n_cols = k->n_cols;
  *n_constraints = k->n_constraints;
  *n_params = k->n_params;
  return CS_OK;
}

extern "C" cs_status cs_rtc_release(void* handle) {
  if (handle == nullptr) return CS_OK;
  RtcKernel* k = static_cast<RtcKernel*>(handle);
  cudaError_t e = cudaLibraryUnload(k->lib);
  delete k;
  if (e != cudaSuccess) return from_cuda(e, "rtc_release");
  return CS_OK;
}

extern "C" cs_status cs_rtc_air_composition(void* handle, const uint32_t* const* h_cols, const uint32_t* h_rc,
                                            const uint32_t* h_params, uint32_t eval_log, uint32_t trace_log,
                                            uint32_t* const h_accum[4], cs_stream stream) {
  return cs_rtc_air_composition_subdomain(handle, h_cols, h_rc, h_params, eval_log, trace_log, 0, h_accum, stream);
}

extern "C" cs_status cs_rtc_air_composition_subdomain(void* handle, const uint32_t* const* h_cols,
                                                      const uint32_t* h_rc, const uint32_t* h_params,
                                                      uint32_t eval_log, uint32_t trace_log, uint32_t log_expansion,
                                                      uint32_t* const h_accum[4], cs_stream stream) {
  CS_CHECK_ARG(handle != nullptr && h_accum != nullptr, "rtc_air_composition: null pointer");
  const RtcKernel* k = static_cast<const RtcKernel*>(handle);
  CS_CHECK_ARG(k->n_cols == 0 || h_cols != nullptr, "rtc_air_composition: null column table");
  CS_CHECK_ARG(k->n_constraints == 0 || h_rc != nullptr, "rtc_air_composition: null weights");
  CS_CHECK_ARG(k->n_params == 0 || h_params != nullptr, "rtc_air_composition: null parameters");
  CS_CHECK_ARG(trace_log >= 1 && eval_log >= trace_log && eval_log - trace_log <= 5 && eval_log <= 30,
               "rtc_air_composition: bad sizes eval %u trace %u", eval_log, trace_log);
  CS_CHECK_ARG(log_expansion <= 8 && eval_log + log_expansion <= 30,
               "rtc_air_composition: bad log_expansion %u for eval %u", log_expansion, eval_log);
  for (uint32_t c = 0; c < k->n_cols; c++) CS_CHECK_ARG(h_cols[c] != nullptr, "rtc_air_composition: column %u is null", c);
  for (int c = 0; c < 4; c++) CS_CHECK_ARG(h_accum[c] != nullptr, "rtc_air_composition: null accumulator");
  // one staging buffer: column pointers, then the weights, the parameters and 1 / V_trace
  // (bit-reversed over the 2^(eval - trace) cosets, component_prover.rs:101-108). The evaluation
  // domain is CanonicCoset(eval + log_expansion).circle_domain().split(log_expansion).0: the
  // half coset keeps the larger domain's initial point G_2^(eval + log_expansion + 1) and takes
  // the step G_2^(eval - 1) (CircleDomain::split; log_expansion 0 is CanonicCoset(eval) itself).
  const size_t n_words = 2 * (size_t)k->n_cols + 4 * (size_t)k->n_constraints + 4 * (size_t)k->n_params + 32;
  std::vector<uint32_t> host(n_words, 0);
  for (uint32_t c = 0; c < k->n_cols; c++) {
    const uint64_t ptr = reinterpret_cast<uint64_t>(h_cols[c]);
    host[2 * c] = (uint32_t)ptr;
    host[2 * c + 1] = (uint32_t)(ptr >> 32);
  }
  uint32_t* w = host.data() + 2 * k->n_cols;
  for (size_t i = 0; i < 4 * (size_t)k->n_constraints; i++) *w++ = h_rc[i] % P;
  for (size_t i = 0; i < 4 * (size_t)k->n_params; i++) *w++ = h_params[i] % P;
  const uint32_t log_expand = eval_log - trace_log;
  for (uint32_t i = 0; i < (1u << log_expand); i++) {
    const uint32_t idx = (subgroup_gen(eval_log + log_expansion + 1) + i * subgroup_gen(eval_log - 1)) & 0x7fffffffu;
    uint32_t x = rtc_point_at(idx).x;
    for (uint32_t t = 1; t < trace_log; t++) x = m31_sub(m31_add(m31_sqr(x), m31_sqr(x)), 1);
    uint32_t j = 0;
    for (uint32_t b = 0; b < log_expand; b++) j |= ((i >> b) & 1u) << (log_expand - 1 - b);
    w[j] = m31_inv(x);
  }
  cudaStream_t st = to_stream(stream);
  uint32_t* dev = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&dev), sizeof(uint32_t) * n_words, st));
  cs_status result = CS_OK;
  cudaError_t e = cudaMemcpyAsync(dev, host.data(), sizeof(uint32_t) * n_words, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const uint32_t* const* cols = reinterpret_cast<const uint32_t* const*>(dev);
    const uint32_t* rc = dev + 2 * k->n_cols;
    const uint32_t* params = rc + 4 * k->n_constraints;
    const uint32_t* den = params + 4 * k->n_params;
    uint32_t* a0 = h_accum[0];
    uint32_t* a1 = h_accum[1];
    uint32_t* a2 = h_accum[2];
    uint32_t* a3 = h_accum[3];
    void* args[] = {&cols, &rc, &params, &den, &eval_log, &trace_log, &a0, &a1, &a2, &a3};
    const uint32_t n = 1u << eval_log;
    const uint32_t blocks = std::max(1u, std::min((n + 255) / 256, 152u * 8));
    e = cudaLaunchKernel(reinterpret_cast<const void*>(k->fn), dim3(blocks), dim3(256), args, 0, st);
    note_launch();
  }
  if (e != cudaSuccess) result = from_cuda(e, "rtc_air_composition");
  const cudaError_t ef = cudaFreeAsync(dev, st);
  if (result == CS_OK && ef != cudaSuccess) return from_cuda(ef, "cudaFreeAsync");
  return result;
}
