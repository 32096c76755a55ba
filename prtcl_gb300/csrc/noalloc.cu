// Field upload that allocates no device memory.
//
// The ordinary upload (upload_varying in model.cu) stages the host bytes of
// real[3] and real[3][3] fields in a temporary device buffer taken from the
// stream-ordered allocator, then spreads them into the field's device layout
// (16-byte padded vectors, planar matrices).  Some callers cannot allocate at
// that point: a host that pre-reserves all device memory for its own pool
// (the allocator call would fail or would fragment it), or a caller that
// must not touch the allocator inside a time-critical section where an
// allocation could block on the device.  This variant stages through a
// fixed, statically sized device array instead.
//
// The array below is one per process and device.  Its device address is
// looked up once per device, and the module that holds it and the staging
// kernels is loaded then too (the runtime loads modules lazily): model
// creation does both for the device current at that time (noalloc_prepare),
// so a host that then hands all remaining device memory to its own pool
// still finds the array resident.  A model used on another device does it on
// its first call there.  Calls are synchronous (each returns after its
// stream has finished with the array) and so cannot be captured into a CUDA
// graph: a call on a capturing stream is refused.
// The array keeps the bytes of the last call; nothing reads it before the
// same call's copy has overwritten the part it uses, so nothing in it has to
// start at zero.  Two calls that overlap in time (from two host threads, on
// any streams) race on the array: serialise them.
#include "model.hpp"

#include <mutex>
#include <vector>

namespace prtcl_gpu {

namespace {

// 8 MiB: 699,050 items of a real[3] field, 233,016 of a real[3][3] field
constexpr size_t kStageBytes = size_t(8) << 20;

__device__ __align__(256) unsigned char g_noalloc_stage[kStageBytes];

std::mutex g_stage_mu;
std::vector<void *> g_stage_addr; // per device, looked up on first use

void *stage_address() {
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_stage_mu);
  if (size_t(dev) >= g_stage_addr.size()) g_stage_addr.resize(size_t(dev) + 1, nullptr);
  if (!g_stage_addr[size_t(dev)]) {
    void *p = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_stage);
    if (rc != cudaSuccess || !p)
      throw Error(std::string("no-alloc upload: cudaGetSymbolAddress failed: ") + cudaGetErrorString(rc));
    g_stage_addr[size_t(dev)] = p;
  }
  return g_stage_addr[size_t(dev)];
}

// the same layouts the ordinary upload writes: vectors padded to float4,
// matrices as nine planes of `cap` floats
__global__ void k_stage_vec3(float const *__restrict__ stage, float4 *__restrict__ dst, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) dst[i] = make_float4(stage[3 * i], stage[3 * i + 1], stage[3 * i + 2], 0.0f);
}
__global__ void k_stage_planar9(float const *__restrict__ stage, float *__restrict__ dst, size_t n, size_t cap) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n)
    for (int k = 0; k < 9; ++k) dst[k * cap + i] = stage[9 * i + k];
}

} // namespace

size_t noalloc_stage_bytes() { return kStageBytes; }

void noalloc_prepare() {
  stage_address();
  cudaFuncAttributes a;
  PG_CUDA(cudaFuncGetAttributes(&a, k_stage_vec3));
  PG_CUDA(cudaFuncGetAttributes(&a, k_stage_planar9));
}

void upload_varying_noalloc(VaryingField &f, size_t count, void const *host, size_t n_items, cudaStream_t s) {
  if (n_items != count)
    throw Error("upload: item count " + std::to_string(n_items) + " != group count " + std::to_string(count));
  size_t hbytes = count * f.type.host_item_bytes();
  bool staged = f.type.is_vec3() || f.type.is_mat3();
  if (staged && hbytes > kStageBytes)
    throw Error("no-alloc upload: " + std::to_string(count) + " items of " + std::to_string(f.type.host_item_bytes()) +
                " bytes need " + std::to_string(hbytes) + " staging bytes, more than the fixed " +
                std::to_string(kStageBytes) + "; use prtcl_gpu_field_upload");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  PG_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    throw Error("no-alloc upload: the stream is being captured; the call is synchronous and cannot be captured");
  void *stage = staged ? stage_address() : nullptr;
  f.version++;
  if (count == 0) return;
  if (!staged) {
    PG_CUDA(cudaMemcpyAsync(f.d, host, hbytes, cudaMemcpyHostToDevice, s));
  } else {
    PG_CUDA(cudaMemcpyAsync(stage, host, hbytes, cudaMemcpyHostToDevice, s));
    if (f.type.is_vec3())
      k_stage_vec3<<<div_up(count, 256), 256, 0, s>>>(static_cast<float const *>(stage), static_cast<float4 *>(f.d),
                                                      count);
    else
      k_stage_planar9<<<div_up(count, 256), 256, 0, s>>>(static_cast<float const *>(stage),
                                                         static_cast<float *>(f.d), count, f.cap);
    count_launch();
    PG_LAUNCH_CHECK();
  }
  PG_CUDA(cudaStreamSynchronize(s));
}

} // namespace prtcl_gpu
