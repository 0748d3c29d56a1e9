// Internal state of the sfx C ABI: meshes, forms and their device buffers.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "sfx.h"

namespace sfx_impl {

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

#define SFX_CUDA_TRY(call)                                                            \
  do {                                                                                \
    cudaError_t err_ = (call);                                                        \
    if (err_ != cudaSuccess)                                                          \
      return ::sfx_impl::fail(SFX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_)); \
  } while (0)

/// Owning device buffer (cudaMalloc / cudaFree).
template <typename T>
struct DeviceBuf {
  T* p = nullptr;
  size_t n = 0;
  DeviceBuf() = default;
  DeviceBuf(const DeviceBuf&) = delete;
  DeviceBuf& operator=(const DeviceBuf&) = delete;
  DeviceBuf(DeviceBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DeviceBuf& operator=(DeviceBuf&& o) noexcept {
    std::swap(p, o.p);
    std::swap(n, o.n);
    return *this;
  }
  ~DeviceBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    reset();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
  cudaError_t upload(const T* host, size_t count) {
    cudaError_t e = alloc(count);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpy(p, host, count * sizeof(T), cudaMemcpyHostToDevice);
  }
};

struct DomainIntegral {
  int material = 0;
  int nparams = 0;
  int state_doubles = 0;  // per quadrature point
  DeviceBuf<double> params;  // [e][nparams]
  DeviceBuf<double> state;   // SoA [k][e*nq+q]
  // stored q-function derivative (stored-tangent Jacobian action)
  DeviceBuf<double> D64;
  DeviceBuf<float> D32;
  DeviceBuf<__half> D16;  // FP16 copy for the FP32 action when the form stores it (tangent16)
  int tangent_rows = 0, tangent_cols = 0;
};

struct BoundaryIntegral {
  int material = 0;
  std::vector<double> params;   // uniform material parameters (host; the q-function is built on the host)
  int64_t num_faces = 0;
  DeviceBuf<int32_t> fconn;     // [f][(p+1)^2] node ids
  DeviceBuf<double> fgeom;      // FGEOM_STRIDE x nq_total
  DeviceBuf<double> Xf;         // [f][3][4] face vertex coordinates (reference configuration)
  DeviceBuf<int32_t> node_ptr;  // over the distinct face nodes (compact list)
  DeviceBuf<int32_t> node_ids;  // global node of each compact entry
  DeviceBuf<int32_t> node_ent;  // (f * npf + local) entries, face order
  int64_t num_face_nodes = 0;
};

/// A domain quantity-of-interest integral (Functional<double(...)>): a
/// built-in integrand kind with uniform parameters.
struct QoiIntegral {
  int kind = 0;
  std::vector<double> params;
};

}  // namespace sfx_impl

struct sfx_mesh_s {
  int nx = 0, ny = 0, nz = 0;
  std::vector<double> vertices;
};

namespace sfx_impl {
/// An int in mapped pinned host memory that kernels can set (device pointer)
/// and the host can read without synchronising: the error flag of the
/// bounded waits in the bulk-copy kernels.
struct MappedFlag {
  int* host = nullptr;
  int* dev = nullptr;
  MappedFlag() = default;
  MappedFlag(const MappedFlag&) = delete;
  MappedFlag& operator=(const MappedFlag&) = delete;
  ~MappedFlag() {
    if (host) cudaFreeHost(host);
  }
  cudaError_t init() {
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&host), sizeof(int), cudaHostAllocMapped);
    if (e != cudaSuccess) return e;
    *host = 0;
    return cudaHostGetDevicePointer(reinterpret_cast<void**>(&dev), host, 0);
  }
  bool raised() const { return host && *static_cast<volatile int*>(host) != 0; }
  void clear() {
    if (host) *static_cast<volatile int*>(host) = 0;
  }
};
/// Streams, events and device vectors of the Jacobian action between host
/// buffers (sfx_jvp_host), created on its first call.
struct HostPipe {
  static constexpr int kMaxChunks = 8;
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t entry = nullptr;  // the caller's stream at the call: the copies start after its earlier work
  cudaEvent_t in_ready[kMaxChunks] = {};
  cudaEvent_t out_ready[kMaxChunks] = {};
  int nevents = 0;
  DeviceBuf<double> du, dr;
  HostPipe() = default;
  HostPipe(const HostPipe&) = delete;
  HostPipe& operator=(const HostPipe&) = delete;
  ~HostPipe() {
    for (int i = 0; i < nevents; i++) {
      cudaEventDestroy(in_ready[i]);
      cudaEventDestroy(out_ready[i]);
    }
    if (entry) cudaEventDestroy(entry);
    if (h2d) cudaStreamDestroy(h2d);
    if (d2h) cudaStreamDestroy(d2h);
  }
};
}  // namespace sfx_impl

struct sfx_form_s {
  sfx_mesh_s mesh;
  sfx_impl::MappedFlag wait_error;  // set by a bulk-copy kernel whose bounded wait expired
  int p = 0, c = 0, Q = 0, NQ = 0, NPE = 0;
  int64_t ne = 0, nnodes = 0, ndofs = 0;
  sfx_impl::DeviceBuf<int32_t> conn;      // [e][NPE]
  sfx_impl::DeviceBuf<int32_t> node_ptr;  // [nnodes + 1]
  sfx_impl::DeviceBuf<int32_t> node_ent;  // e * NPE + local, element order
  sfx_impl::DeviceBuf<double> geom64;
  sfx_impl::DeviceBuf<float> geom32;
  sfx_impl::DeviceBuf<double> Xe;     // [e][3][8] element vertex coordinates (reference configuration)
  sfx_impl::DeviceBuf<double> shape;  // shape displacement [3][nnodes] when has_shape
  bool has_shape = false;
  sfx_impl::DeviceBuf<double> e64;  // E-vector scratch
  sfx_impl::DeviceBuf<float> e32;
  sfx_impl::DeviceBuf<double> ef64;  // face E-vector scratch
  sfx_impl::DeviceBuf<float> ef32;
  sfx_impl::DeviceBuf<double> u_lin64;
  sfx_impl::DeviceBuf<float> u_lin32;
  double t_lin = 0.0;
  bool linearized = false;
  bool update_qdata = false;
  int jvp_mode = SFX_JVP_STORED_TANGENT;
  bool tangent16 = false;  // the FP32 action streams an FP16 copy of the tangent
  // forms built from an imported element table (sfx_form_create_from_table):
  // host copies of the tables and the scalar adjacency of the CSR graph
  bool general = false;
  std::vector<int32_t> conn_host;  // [e][NPE]
  std::vector<double> Xe_host;     // [e][3][8]
  sfx_impl::DeviceBuf<int64_t> sptr;
  sfx_impl::DeviceBuf<int32_t> scol;
  std::vector<sfx_impl::DomainIntegral> domain;
  std::vector<sfx_impl::BoundaryIntegral> boundary;
  std::vector<sfx_impl::BoundaryIntegral> face_sets;  // faces for integrals evaluated by the caller's kernels
  // quantity of interest (test space QOI): integrals and the per-element /
  // per-face value scratch of its deterministic sum
  bool qoi = false;
  std::vector<sfx_impl::QoiIntegral> qoi_domain;
  std::vector<sfx_impl::BoundaryIntegral> qoi_boundary;  // material = QoI kind
  sfx_impl::DeviceBuf<double> qoi_vals;
  sfx_impl::DeviceBuf<double> qoi_partial;
  // shape-sensitivity E-vectors [e][3][node] and [face][3][node]
  sfx_impl::DeviceBuf<double> eshape;
  sfx_impl::DeviceBuf<double> efshape;
  // CSR graph (built on first request)
  bool csr_built = false;
  int64_t nnz = 0;
  sfx_impl::DeviceBuf<int64_t> row_ptr;
  sfx_impl::DeviceBuf<int32_t> col;
  sfx_impl::DeviceBuf<double> ke;  // element matrices scratch
  sfx_impl::DeviceBuf<double> kf;  // face matrices scratch
  sfx_impl::HostPipe host_pipe;    // sfx_jvp_host
};
