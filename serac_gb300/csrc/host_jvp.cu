// sfx_jvp_host: the FP64 Jacobian action between host buffers, with the
// host <-> device copies overlapped with the kernels.
//
// Structured meshes number elements e = ex + nx (ey + ny ez) and nodes
// x + Nx (y + Ny z), so a slab of element layers [L0, L1) reads the node
// planes [p L0, p L1] and, once every slab up to it is done, completes the
// node planes [p L0, p L1) (plane p L1 also belongs to layer L1).  Slab k is
// therefore copied in on one stream (which first waits for the caller's
// stream), computed on the caller's stream after its copy event, and its
// completed planes are copied out on a third stream after its compute event,
// while slab k + 1 is being copied in.  Every
// kernel and the order of every sum are those of sfx_jvp, so the result is
// bitwise the same.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "dispatch.hpp"
#include "form.hpp"
#include "sfx.h"

using namespace sfx_impl;

namespace {

int ensure_pipe(sfx_form_s& f, int chunks) {
  HostPipe& hp = f.host_pipe;
  if (!hp.h2d) SFX_CUDA_TRY(cudaStreamCreateWithFlags(&hp.h2d, cudaStreamNonBlocking));
  if (!hp.d2h) SFX_CUDA_TRY(cudaStreamCreateWithFlags(&hp.d2h, cudaStreamNonBlocking));
  if (!hp.entry) SFX_CUDA_TRY(cudaEventCreateWithFlags(&hp.entry, cudaEventDisableTiming));
  while (hp.nevents < chunks) {
    SFX_CUDA_TRY(cudaEventCreateWithFlags(&hp.in_ready[hp.nevents], cudaEventDisableTiming));
    if (cudaEventCreateWithFlags(&hp.out_ready[hp.nevents], cudaEventDisableTiming) != cudaSuccess) {
      cudaEventDestroy(hp.in_ready[hp.nevents]);
      return fail(SFX_ERR_CUDA, "event creation failed");
    }
    hp.nevents++;
  }
  const size_t n = size_t(f.ndofs);
  if (hp.du.n < n && hp.du.alloc(n) != cudaSuccess) return fail(SFX_ERR_NOMEM, "host-action input vector");
  if (hp.dr.n < n && hp.dr.alloc(n) != cudaSuccess) return fail(SFX_ERR_NOMEM, "host-action output vector");
  return SFX_OK;
}

/// node planes [z0, z1) of every component, between host and device
int copy_planes(const sfx_form_s& f, double* dst, const double* src, int64_t z0, int64_t z1, cudaMemcpyKind kind,
                cudaStream_t s) {
  if (z1 <= z0) return SFX_OK;
  const int64_t plane = (int64_t(f.p) * f.mesh.nx + 1) * (int64_t(f.p) * f.mesh.ny + 1);
  const size_t bytes = size_t((z1 - z0) * plane) * sizeof(double);
  for (int c = 0; c < f.c; c++) {
    const int64_t off = c * f.nnodes + z0 * plane;
    SFX_CUDA_TRY(cudaMemcpyAsync(dst + off, src + off, bytes, kind, s));
  }
  return SFX_OK;
}

bool pipelined(const sfx_form_s& f) {
  return !f.general && !f.qoi && f.domain.size() == 1 && f.boundary.empty() &&
         f.jvp_mode == SFX_JVP_STORED_TANGENT && f.mesh.nz >= 1;
}

}  // namespace

extern "C" int sfx_jvp_host(sfx_form form, const double* du, double* dr, void* stream) {
  if (!form) return fail(SFX_ERR_INVALID, "null form");
  if (!du || !dr) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp_host");
  sfx_form_s& f = *form;
  auto s = static_cast<cudaStream_t>(stream);
  const int chunks = pipelined(f) ? std::min(f.mesh.nz, HostPipe::kMaxChunks) : 0;
  if (int rc = ensure_pipe(f, std::max(chunks, 1))) return rc;
  HostPipe& hp = f.host_pipe;
  const size_t bytes = size_t(f.ndofs) * sizeof(double);
  if (chunks == 0) {
    SFX_CUDA_TRY(cudaMemcpyAsync(hp.du.p, du, bytes, cudaMemcpyHostToDevice, s));
    if (int rc = sfx_jvp(form, hp.du.p, hp.dr.p, stream)) return rc;
    SFX_CUDA_TRY(cudaMemcpyAsync(dr, hp.dr.p, bytes, cudaMemcpyDeviceToHost, s));
    SFX_CUDA_TRY(cudaStreamSynchronize(s));
    return SFX_OK;
  }
  SFX_CUDA_TRY(cudaEventRecord(hp.entry, s));
  SFX_CUDA_TRY(cudaStreamWaitEvent(hp.h2d, hp.entry, 0));
  const int64_t nz = f.mesh.nz, layer = int64_t(f.mesh.nx) * f.mesh.ny, p = f.p;
  const int64_t Nz = p * nz + 1;
  const int64_t plane = (p * f.mesh.nx + 1) * (p * f.mesh.ny + 1);
  for (int k = 0; k < chunks; k++) {
    const int64_t L0 = nz * k / chunks, L1 = nz * (k + 1) / chunks;
    // in: the planes up to and including p L1 not sent before
    const int64_t in0 = k == 0 ? 0 : p * L0 + 1, in1 = p * L1 + 1;
    if (int rc = copy_planes(f, hp.du.p, du, in0, in1, cudaMemcpyHostToDevice, hp.h2d)) return rc;
    SFX_CUDA_TRY(cudaEventRecord(hp.in_ready[k], hp.h2d));
    SFX_CUDA_TRY(cudaStreamWaitEvent(s, hp.in_ready[k], 0));
    if (int rc = launch_jvp_stored_range(f, f.domain[0], hp.du.p, f.e64.p, L0 * layer, L1 * layer, s)) return rc;
    // out: the planes this slab completes (the last slab: through the top)
    const int64_t out0 = p * L0, out1 = k == chunks - 1 ? Nz : p * L1;
    if (int rc = scatter_evector_range(f, f.e64.p, hp.dr.p, out0 * plane, out1 * plane, s)) return rc;
    SFX_CUDA_TRY(cudaEventRecord(hp.out_ready[k], s));
    SFX_CUDA_TRY(cudaStreamWaitEvent(hp.d2h, hp.out_ready[k], 0));
    if (int rc = copy_planes(f, dr, hp.dr.p, out0, out1, cudaMemcpyDeviceToHost, hp.d2h)) return rc;
  }
  SFX_CUDA_TRY(cudaStreamSynchronize(hp.d2h));
  SFX_CUDA_TRY(cudaStreamSynchronize(s));
  return SFX_OK;
}
