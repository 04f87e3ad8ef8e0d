// L2 read-bandwidth probe: the denominator of the traversal roofline.
//
// Traversal reads BVH nodes and leaf slots that stay resident in the 129 MB
// L2 once a scene is warm, so its bandwidth ceiling is the L2's, not HBM's.
// This kernel measures that ceiling on the GPU at hand: each block reads its
// own chunk of a working set smaller than L2, over and over, with 16-byte
// loads that bypass L1 (ld.global.cg).  The loads use immediate offsets from
// one base address and each feeds a single XOR, so the probe is bound by the
// memory system and not by instruction issue.  Bytes counted = working set x
// repeats; the launch is timed with CUDA events.
//
// Measurement code only: it is built into its own library
// (libbling_probe.so), not into the renderer's C ABI.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kThreads = 512;
constexpr int kUnroll = 8;

__global__ void __launch_bounds__(kThreads) k_l2_read(const uint4* __restrict__ buf,
                                                      size_t chunk16, int repeats,
                                                      uint32_t* __restrict__ sink) {
  const uint4* base = buf + (size_t)blockIdx.x * chunk16 + threadIdx.x;
  uint32_t acc = 0;
  for (int r = 0; r < repeats; r++) {
    for (size_t k = 0; k < chunk16; k += (size_t)kThreads * kUnroll) {
      const uint4* p = base + k;
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        uint32_t x, y, z, w;
        asm volatile("ld.global.cg.v4.u32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(x), "=r"(y), "=r"(z), "=r"(w)
                     : "l"(p + u * kThreads));
        acc ^= x ^ w;
      }
    }
  }
  sink[(size_t)blockIdx.x * kThreads + threadIdx.x] = acc;
}

__global__ void k_fill(uint4* buf, size_t n16) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16;
       i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_uint4((uint32_t)i, (uint32_t)(i >> 7), 0x9e3779b9u, (uint32_t)i * 3u);
}

}  // namespace

extern "C" {

// Measures L2 read bandwidth in GB/s over a working set of about `bytes`,
// read `repeats` times by `blocks_per_sm` x SM-count blocks of 512 threads;
// each block reads a chunk of its own (a multiple of 512 x 8 x 16 bytes).
// Writes the timed launch's duration to *out_ms and the working set actually
// used to *out_bytes.  Returns a negative value on a CUDA error or bad
// argument.  Allocates and frees its own buffers.
double bling_probe_l2_read_gbs(int device, size_t bytes, int repeats, int blocks_per_sm,
                               float* out_ms, size_t* out_bytes) {
  if (cudaSetDevice(device) != cudaSuccess) return -1.0;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return -1.0;
  if (blocks_per_sm <= 0 || blocks_per_sm > 4 || repeats <= 0) return -2.0;
  const size_t blocks = (size_t)sms * blocks_per_sm;
  const size_t step = (size_t)kThreads * kUnroll;
  size_t chunk16 = bytes / 16 / blocks;
  chunk16 -= chunk16 % step;
  if (chunk16 == 0) return -2.0;
  const size_t n16 = chunk16 * blocks;
  uint4* buf = nullptr;
  uint32_t* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double gbs = -1.0;
  if (cudaMalloc(&buf, n16 * 16) != cudaSuccess) return -1.0;
  if (cudaMalloc(&sink, blocks * kThreads * 4) != cudaSuccess) {
    cudaFree(buf);
    return -1.0;
  }
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fill<<<sms * 4, 256>>>(buf, n16);
  // warm the L2 with the working set, then time
  k_l2_read<<<(unsigned)blocks, kThreads>>>(buf, chunk16, 2, sink);
  cudaEventRecord(e0);
  k_l2_read<<<(unsigned)blocks, kThreads>>>(buf, chunk16, repeats, sink);
  cudaEventRecord(e1);
  if (cudaEventSynchronize(e1) == cudaSuccess) {
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (out_ms) *out_ms = ms;
    if (out_bytes) *out_bytes = n16 * 16;
    gbs = (double)n16 * 16.0 * repeats / (ms * 1e-3) / 1e9;
  }
  if (cudaGetLastError() != cudaSuccess) gbs = -1.0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  cudaFree(buf);
  return gbs;
}

}  // extern "C"
