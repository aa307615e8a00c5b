// capi_util.h -- helpers shared by the C-ABI translation units: the
// thread-local last-error string, CUDA error checks that throw, the guard
// that turns exceptions into return codes, and a device buffer.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <stdexcept>
#include <string>

#include "../../include/swift_gb300.h"

namespace sphgpu {
namespace capi {

extern thread_local std::string g_err;

inline int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      throw sphgpu::capi::CudaError(std::string(#call) + ": " +               \
                                    cudaGetErrorString(e_));                  \
  } while (0)

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    release();
    n = count;
    if (count == 0) count = 1;
    CK(cudaMalloc(&p, count * sizeof(T)));
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    if (count > n) alloc(count);
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
};

inline int guard(const std::function<int()>& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    cudaGetLastError();  // a reported non-sticky error must not reach the next check
    return fail(SPHGPU_ECUDA, e.what());
  } catch (const std::bad_alloc&) {
    return fail(SPHGPU_ENOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    const std::string m = e.what();
    if (m.find("no CUDA device") != std::string::npos) return fail(SPHGPU_ENODEV, m);
    return fail(SPHGPU_EINVAL, m);
  }
}

}  // namespace capi
}  // namespace sphgpu
