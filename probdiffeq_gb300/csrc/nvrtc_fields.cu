// User vector fields compiled at run time (NVRTC) into the isotropic solver.
//
// The reference takes any Python callable as the vector field
// (probdiffeq.ode, _probdiffeq/problems.py:283-295) and traces it into the
// solver.  Here a field is CUDA C++ source of a functor
//
//   struct Field {
//     static constexpr int D = ...;   // state dimension
//     static constexpr int P = ...;   // number of parameters
//     template <typename S, typename T>
//     PDQ_HD static void eval(const S* u, const T* p, S* out);  // out = f(u; p)
//   };
//
// written generically over the scalar S (float, double, Taylor jets, dual
// numbers: +, -, * and multiplication / division by parameters), exactly
// like the built-in fields, so one definition yields f, its Jacobian (the
// dense TS1 linearisation) and the Taylor-mode initial derivatives.
// pdq_register_field compiles the source with the solver templates (headers
// embedded in this library) for sm_103a and reports compiler errors; each
// variant of the isotropic kernel (precision, nu, interpolation, strategy)
// and of the dense one (precision, nu, TS0/TS1, strategy) is compiled and
// loaded on first use and cached.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "pdq_nvtx.h"
#include "bd_launch.cuh"
#include "dense_solver.cuh"
#include "iso_solver.cuh"
#include "lml_adjoint.cuh"
#include "nvrtc_fields.h"
#include "pdq.h"
#include "pdq_embedded_headers.inc"  // kPdqHeaderCount, kPdqHeaderNames, kPdqHeaderSources (generated)

namespace {

struct UserField {
  std::string name, source;
  int dim = 0, params = 0;
  bool stencil = false;  // a block-diagonal stencil (struct Stencil) rather than a field (struct Field)
  std::mutex mu;
  // (kernel expression) -> loaded kernel
  std::map<std::string, cudaKernel_t> kernels;
  std::vector<cudaLibrary_t> libraries;
};

std::mutex g_registry_mu;
std::vector<std::unique_ptr<UserField>> g_fields;

UserField* lookup(int32_t field) {
  std::lock_guard<std::mutex> lock(g_registry_mu);
  const int64_t k = int64_t(field) - PDQ_FIELD_USER_BASE;
  if (k < 0 || k >= int64_t(g_fields.size())) return nullptr;
  return g_fields[size_t(k)].get();
}

const char* tf(bool b) { return b ? "true" : "false"; }

// gen: the instantiation with TS1 / error_state_std / damping; the filter
// without them and with exact landings takes the branch-light lean kernel
// (as the built-in fields' dispatch)
std::string kernel_expression(bool f64, int nu, bool interp, bool fp, bool gen) {
  if (!interp && !fp && !gen)
    return std::string("pdq::iso_lean_kernel<") + (f64 ? "double" : "float") + ", " + std::to_string(nu) +
           ", pdq_user::Field>";
  return std::string("pdq::iso_adaptive_kernel<") + (f64 ? "double" : "float") + ", " + std::to_string(nu) +
         ", pdq_user::Field, " + tf(interp) + ", " + tf(fp) + ", " + tf(gen) + ">";
}

std::string dense_expression(bool f64, int nu, bool ts1, bool fp) {
  return std::string("pdq::dense_adaptive_kernel<") + (f64 ? "double" : "float") + ", " + std::to_string(nu) +
         ", pdq_user::Field, " + tf(ts1) + ", " + tf(fp) + ">";
}

std::string bd_expression(bool f64, int nu, bool fp) {
  return std::string("pdq::bd_adaptive_kernel<") + (f64 ? "double" : "float") + ", " + std::to_string(nu) + ", " +
         tf(fp) + ", pdq_user::Stencil>";
}

// The LML kernels of a user field: the covariance plan (field-independent,
// compiled into the same module) and the per-sample kernels.
std::vector<std::string> lml_expressions(bool f64, int nu, bool adjoint) {
  const std::string T = f64 ? "double" : "float", N = std::to_string(nu);
  std::vector<std::string> e = {"pdq::lml_plan_kernel<" + T + ", " + N + ">"};
  if (adjoint) {
    e.push_back("pdq::lml_adj_fwd_kernel<" + T + ", " + N + ", pdq_user::Field>");
    e.push_back("pdq::lml_adj_bwd_kernel<" + T + ", " + N + ", pdq_user::Field>");
  } else {
    e.push_back("pdq::lml_kernel<" + T + ", " + N + ", pdq_user::Field>");
  }
  return e;
}

void copy_log(const std::string& text, char* log, size_t log_bytes) {
  if (log == nullptr || log_bytes == 0) return;
  const size_t n = text.size() < log_bytes - 1 ? text.size() : log_bytes - 1;
  std::memcpy(log, text.data(), n);
  log[n] = '\0';
}

// Compile the solver templates with the field source; returns the cubin and
// the lowered (mangled) names of the requested kernel instantiations.
pdq_status compile(const std::string& source, const std::vector<std::string>& expressions, std::string* cubin,
                   std::vector<std::string>* lowered, std::string* log, const char* header = "iso_solver.cuh") {
  const std::string program =
      std::string("#include \"") + header + "\"\nnamespace pdq_user {\n" + source + "\n}  // namespace pdq_user\n";
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, program.c_str(), "user_field.cu", kPdqHeaderCount, kPdqHeaderSources,
                         kPdqHeaderNames) != NVRTC_SUCCESS)
    return PDQ_ERROR_COMPILE;
  for (const auto& e : expressions) nvrtcAddNameExpression(prog, e.c_str());
  // -default-device: the kernels' local lambdas (unannotated) are device code
  const char* options[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", "-default-device"};
  const nvrtcResult rc = nvrtcCompileProgram(prog, 4, options);
  size_t log_size = 0;
  nvrtcGetProgramLogSize(prog, &log_size);
  std::string text(log_size, '\0');
  if (log_size > 0) nvrtcGetProgramLog(prog, &text[0]);
  if (log) *log = text;
  if (rc != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return PDQ_ERROR_COMPILE;
  }
  size_t size = 0;
  if (nvrtcGetCUBINSize(prog, &size) != NVRTC_SUCCESS || size == 0) {
    nvrtcDestroyProgram(&prog);
    return PDQ_ERROR_COMPILE;
  }
  cubin->assign(size, '\0');
  nvrtcGetCUBIN(prog, &(*cubin)[0]);
  lowered->clear();
  for (const auto& e : expressions) {
    const char* name = nullptr;
    if (nvrtcGetLoweredName(prog, e.c_str(), &name) != NVRTC_SUCCESS || name == nullptr) {
      nvrtcDestroyProgram(&prog);
      return PDQ_ERROR_COMPILE;
    }
    lowered->emplace_back(name);
  }
  nvrtcDestroyProgram(&prog);
  return PDQ_SUCCESS;
}

bool nonempty(const char* s) { return s != nullptr && s[0] != '\0'; }

}  // namespace

extern "C" pdq_status pdq_register_field(const char* name, const char* source, int32_t dim, int32_t num_params,
                                         int32_t* field_id, char* log, size_t log_bytes) {
  pdq::NvtxRange nvtx_range("pdq_register_field");
  if (field_id == nullptr || !nonempty(name) || !nonempty(source) ||
      dim < 1 || dim > 64 || num_params < 0 || num_params > 64)
    return PDQ_ERROR_INVALID_VALUE;
  // validate by compiling one variant (no device needed)
  std::string cubin, text;
  std::vector<std::string> lowered;
  const pdq_status st =
      compile(source, {kernel_expression(false, 2, false, false, false)}, &cubin, &lowered, &text, "iso_lean.cuh");
  copy_log(text, log, log_bytes);
  if (st != PDQ_SUCCESS) return st;
  auto f = std::make_unique<UserField>();
  f->name = name;
  f->source = source;
  f->dim = dim;
  f->params = num_params;
  std::lock_guard<std::mutex> lock(g_registry_mu);
  *field_id = PDQ_FIELD_USER_BASE + int32_t(g_fields.size());
  g_fields.push_back(std::move(f));
  return PDQ_SUCCESS;
}

extern "C" pdq_status pdq_register_stencil(const char* name, const char* source, int32_t num_params,
                                           int32_t* field_id, char* log, size_t log_bytes) {
  pdq::NvtxRange nvtx_range("pdq_register_stencil");
  if (field_id == nullptr || !nonempty(name) || !nonempty(source) || num_params < 0 || num_params > 64)
    return PDQ_ERROR_INVALID_VALUE;
  std::string cubin, text;
  std::vector<std::string> lowered;
  const pdq_status st = compile(source, {bd_expression(false, 3, false)}, &cubin, &lowered, &text, "bd_solver.cuh");
  copy_log(text, log, log_bytes);
  if (st != PDQ_SUCCESS) return st;
  auto f = std::make_unique<UserField>();
  f->name = name;
  f->source = source;
  f->dim = -1;  // any d
  f->params = num_params;
  f->stencil = true;
  std::lock_guard<std::mutex> lock(g_registry_mu);
  *field_id = PDQ_FIELD_USER_BASE + int32_t(g_fields.size());
  g_fields.push_back(std::move(f));
  return PDQ_SUCCESS;
}

int pdq_user_field_dim(int32_t field) {
  UserField* f = lookup(field);
  return f ? f->dim : 0;
}

bool pdq_user_field_is_stencil(int32_t field) {
  UserField* f = lookup(field);
  return f != nullptr && f->stencil;
}

int pdq_user_field_params(int32_t field) {
  UserField* f = lookup(field);
  return f ? f->params : -1;
}

namespace {

// The kernel for `expression` (compiled with `header`), loaded on first use.
cudaError_t user_kernel(UserField* f, const std::string& expression, const char* header, cudaKernel_t* kernel) {
  std::lock_guard<std::mutex> lock(f->mu);
  auto it = f->kernels.find(expression);
  if (it != f->kernels.end()) {
    *kernel = it->second;
    return cudaSuccess;
  }
  std::string cubin, text;
  std::vector<std::string> lowered;
  if (compile(f->source, {expression}, &cubin, &lowered, &text, header) != PDQ_SUCCESS) return cudaErrorInvalidSource;
  cudaLibrary_t lib = nullptr;
  cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) return e;
  e = cudaLibraryGetKernel(kernel, lib, lowered[0].c_str());
  if (e != cudaSuccess) return e;
  // the per-thread stack limit must cover the kernel's frame (as for the built-in kernels)
  cudaFuncAttributes attr;
  e = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(*kernel));
  if (e != cudaSuccess) return e;
  size_t cur = 0;
  e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
  if (e != cudaSuccess) return e;
  if (attr.localSizeBytes + 1024 > cur) {
    e = cudaDeviceSetLimit(cudaLimitStackSize, attr.localSizeBytes + 1024);
    if (e != cudaSuccess) return e;
  }
  f->libraries.push_back(lib);
  f->kernels.emplace(expression, *kernel);
  return cudaSuccess;
}

// The kernels for `expressions` (one module compiled with `header`), loaded on first use.
cudaError_t user_kernels(UserField* f, const std::vector<std::string>& expressions, const char* header,
                         std::vector<cudaKernel_t>* out) {
  std::lock_guard<std::mutex> lock(f->mu);
  out->clear();
  bool all = true;
  for (const auto& e : expressions) {
    auto it = f->kernels.find(e);
    if (it == f->kernels.end()) {
      all = false;
      break;
    }
    out->push_back(it->second);
  }
  if (all) return cudaSuccess;
  out->clear();
  std::string cubin, text;
  std::vector<std::string> lowered;
  if (compile(f->source, expressions, &cubin, &lowered, &text, header) != PDQ_SUCCESS) return cudaErrorInvalidSource;
  cudaLibrary_t lib = nullptr;
  cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) return e;
  f->libraries.push_back(lib);
  for (size_t i = 0; i < expressions.size(); ++i) {
    cudaKernel_t k = nullptr;
    e = cudaLibraryGetKernel(&k, lib, lowered[i].c_str());
    if (e != cudaSuccess) return e;
    cudaFuncAttributes attr;
    e = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(k));
    if (e != cudaSuccess) return e;
    size_t cur = 0;
    e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
    if (e != cudaSuccess) return e;
    if (attr.localSizeBytes + 1024 > cur) {
      e = cudaDeviceSetLimit(cudaLimitStackSize, attr.localSizeBytes + 1024);
      if (e != cudaSuccess) return e;
    }
    f->kernels.emplace(expressions[i], k);
    out->push_back(k);
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t pdq_launch_iso_user(const pdq::IsoArgs& a, int32_t field, bool f64, int nu, bool interp, bool fp,
                                cudaStream_t stream, int block) {
  UserField* f = lookup(field);
  if (f == nullptr || nu < 1 || nu > 5) return cudaErrorInvalidValue;
  // (the lean instantiation's single-QR update needs TS0 without damping)
  const bool gen = fp || a.ts1 || a.state_error || a.damp != 0.0;
  cudaKernel_t kernel = nullptr;
  cudaError_t e = user_kernel(f, kernel_expression(f64, nu, interp, fp, gen), "iso_lean.cuh", &kernel);
  if (e != cudaSuccess) return e;
  pdq::IsoArgs args = a;
  void* params[] = {&args};
  const unsigned grid = unsigned((a.B + block - 1) / block);
  return cudaLaunchKernel(reinterpret_cast<const void*>(kernel), dim3(grid), dim3(unsigned(block)), params, 0, stream);
}

cudaError_t pdq_launch_dense_user(const pdq::DenseArgs& a, int32_t field, bool f64, int nu, bool ts1, bool fp,
                                  cudaStream_t stream) {
  UserField* f = lookup(field);
  if (f == nullptr || nu < 2 || nu > 3) return cudaErrorInvalidValue;
  cudaKernel_t kernel = nullptr;
  cudaError_t e = user_kernel(f, dense_expression(f64, nu, ts1, fp), "dense_solver.cuh", &kernel);
  if (e != cudaSuccess) return e;
  pdq::DenseArgs args = a;
  void* params[] = {&args};
  const int block = a.instances_per_block > 0 ? a.instances_per_block : 32;  // one thread per instance
  const unsigned grid = unsigned((a.B + block - 1) / block);
  return cudaLaunchKernel(reinterpret_cast<const void*>(kernel), dim3(grid), dim3(unsigned(block)), params, 0, stream);
}

cudaError_t pdq_launch_lml_user(const pdq::LmlArgs& a, int32_t field, bool f64, int nu, cudaStream_t stream) {
  UserField* f = lookup(field);
  if (f == nullptr || nu < 2 || nu > 3) return cudaErrorInvalidValue;
  std::vector<cudaKernel_t> k;
  cudaError_t e = user_kernels(f, lml_expressions(f64, nu, false), "lml_solver.cuh", &k);
  if (e != cudaSuccess) return e;
  pdq::LmlArgs args = a;
  void* params[] = {&args};
  e = cudaLaunchKernel(reinterpret_cast<const void*>(k[0]), dim3(1), dim3(pdq::kLmlPlanThreads), params, 0, stream);
  if (e != cudaSuccess) return e;
  const int64_t threads = a.B * a.lanes_per_sample;
  const unsigned grid = unsigned((threads + pdq::kLmlThreads - 1) / pdq::kLmlThreads);
  return cudaLaunchKernel(reinterpret_cast<const void*>(k[1]), dim3(grid), dim3(pdq::kLmlThreads), params, 0, stream);
}

cudaError_t pdq_launch_lml_adj_user(const pdq::LmlAdjArgs& aa, int32_t field, bool f64, int nu, bool backward,
                                    cudaStream_t stream) {
  UserField* f = lookup(field);
  if (f == nullptr || nu < 2 || nu > 3) return cudaErrorInvalidValue;
  std::vector<cudaKernel_t> k;
  cudaError_t e = user_kernels(f, lml_expressions(f64, nu, true), "lml_adjoint.cuh", &k);
  if (e != cudaSuccess) return e;
  pdq::LmlAdjArgs args = aa;
  void* params[] = {&args};
  const unsigned grid = unsigned((aa.base.B + pdq::kLmlThreads - 1) / pdq::kLmlThreads);
  if (backward)
    return cudaLaunchKernel(reinterpret_cast<const void*>(k[2]), dim3(grid), dim3(pdq::kLmlThreads), params, 0, stream);
  pdq::LmlArgs base = aa.base;
  void* plan_params[] = {&base};
  e = cudaLaunchKernel(reinterpret_cast<const void*>(k[0]), dim3(1), dim3(pdq::kLmlPlanThreads), plan_params, 0, stream);
  if (e != cudaSuccess) return e;
  return cudaLaunchKernel(reinterpret_cast<const void*>(k[1]), dim3(grid), dim3(pdq::kLmlThreads), params, 0, stream);
}

cudaError_t pdq_launch_bd_user(const pdq::BdArgs& a, int32_t field, bool f64, int nu, cudaStream_t stream) {
  UserField* f = lookup(field);
  if (f == nullptr || !f->stencil || nu < 2 || nu > 4) return cudaErrorInvalidValue;
  cudaKernel_t kernel = nullptr;
  cudaError_t e = user_kernel(f, bd_expression(f64, nu, a.fixedpoint != 0), "bd_solver.cuh", &kernel);
  if (e != cudaSuccess) return e;
  // bd_smem_bytes<T, NU>: staged means (n rows), new terms, scales and current scales (3 rows) of dl dimensions
  const size_t smem = size_t(nu + 1 + 3) * size_t(a.d / a.cluster) * (f64 ? sizeof(double) : sizeof(float));
  return pdq::launch_bd_cluster(reinterpret_cast<const void*>(kernel), a, smem, stream);
}
