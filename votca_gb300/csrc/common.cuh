// Shared host/device helpers of the GB300 BSE library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/votca_gb300_bse.h"

namespace vgb {

// Error carried from the C++ core to the C ABI (mapped to a bse_status code).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error(code, msg); }

inline void cuda_check(cudaError_t e, const char *what, const char *file, int line) {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? BSE_ERR_OUT_OF_MEMORY : BSE_ERR_CUDA;
    fail(code, std::string(what) + " failed at " + file + ":" + std::to_string(line) + ": " +
                   cudaGetErrorString(e));
  }
}
#define VGB_CUDA(x) ::vgb::cuda_check((x), #x, __FILE__, __LINE__)
#define VGB_LAUNCH_CHECK() ::vgb::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)
#define VGB_REQUIRE(cond, msg)                                   \
  do {                                                           \
    if (!(cond)) ::vgb::fail(BSE_ERR_ARGUMENT, std::string(msg)); \
  } while (0)

// Stream on which DeviceBuffer allocates and frees on the calling thread (set by
// the C ABI entry points to the handle's stream).  With a stream set, buffers
// use the stream-ordered allocator (cudaMallocAsync / cudaFreeAsync), which does
// not synchronise the device, so independent handles can work concurrently.
cudaStream_t &alloc_stream();
struct AllocStreamScope {
  cudaStream_t saved;
  explicit AllocStreamScope(cudaStream_t s) : saved(alloc_stream()) { alloc_stream() = s; }
  ~AllocStreamScope() { alloc_stream() = saved; }
};
void *device_alloc(size_t bytes, cudaStream_t &used);
void device_free(void *p, cudaStream_t used);
void trim_pool();  // return unused stream-ordered blocks to the driver

// Owning device buffer.
template <typename T>
struct DeviceBuffer {
  T *ptr = nullptr;
  size_t count = 0;
  cudaStream_t stream = nullptr;  // stream of the stream-ordered allocation (null: cudaMalloc)
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t n) { resize(n); }
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  DeviceBuffer(DeviceBuffer &&o) noexcept : ptr(o.ptr), count(o.count), stream(o.stream) {
    o.ptr = nullptr;
    o.count = 0;
  }
  DeviceBuffer &operator=(DeviceBuffer &&o) noexcept {
    if (this != &o) {
      release();
      ptr = o.ptr; count = o.count; stream = o.stream;
      o.ptr = nullptr; o.count = 0;
    }
    return *this;
  }
  ~DeviceBuffer() { release(); }
  void resize(size_t n) {
    if (n <= count && ptr) return;
    release();
    if (n == 0) return;
    ptr = (T *)device_alloc(n * sizeof(T), stream);
    count = n;
  }
  void release() {
    if (ptr) device_free(ptr, stream);
    ptr = nullptr;
    count = 0;
  }
  T *get() const { return ptr; }
  size_t bytes() const { return count * sizeof(T); }
};

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Number of SMs of the current device (152 on GB300).
int sm_count();

// Measured FP64 FMA throughput of the current device in TFLOP/s.
double probe_fp64_tflops();

// Screening (screening.cu)
void rpa_epsilon(const bse_mmn_desc &desc, const double *const *slices, const double *energies,
                 int64_t rpatotal, int64_t homo, int64_t rpamin, int64_t rpamax, double wr, double wi,
                 double eta, double *eps_host, cudaStream_t s);
void cholesky_inverse(int64_t n, const double *a_host, int64_t lda, double *inv_host, int64_t ldi,
                      cudaStream_t s);
void positive_inverse(int64_t n, const double *a_host, int64_t lda, double cutoff, double *inv_host,
                      int64_t ldi, cudaStream_t s);
void mmn_multiply_right(const bse_mmn_desc &desc, double *const *slices, const double *U_host,
                        int64_t ldu, cudaStream_t s);

// Mmn producer (threecenter.cu)
void fill_3c_mo(const bse_mmn_desc &desc, double *const *slices, const double *ao3c, int64_t nbf,
                const double *C, int64_t ldc, int64_t nmo, cudaStream_t s);
void transition_dipoles(const double *ao_dip, int64_t nbf, const double *C, int64_t ldc, int64_t nmo,
                        int64_t vmin, int64_t vtotal, int64_t cmin, int64_t ctotal, const double *X,
                        const double *Y, int64_t ldx, int64_t nstates, double prefactor, bool accumulate,
                        double *dip, cudaStream_t s);
void aux_pseudo_inv_sqrt(int64_t n, const double *V, int64_t ldv, double etol, double *out, int64_t ldo,
                         int64_t *removed, cudaStream_t s);
void aux_pseudo_inv_sqrt_gwbse(int64_t n, const double *S, int64_t lds, const double *V, int64_t ldv,
                               double etol, double *out, int64_t ldo, int64_t *removed, cudaStream_t s);

}  // namespace vgb
