// Kinetic energy and momentum of a caller-owned velocity array, without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need this number: a host
// loop that reserves all the GPU memory it will use up front and must not allocate afterwards
// (an allocation mid-run could stall the loop or fail when memory is fully committed), or an
// embedding framework that owns the device heap and only hands out its own buffers.  For them
// this entry point takes device pointers in and out and keeps its per-block scratch in a fixed
// array that is part of the loaded library.
//
// Scratch: the file-scope __device__ array below, 8,224 doubles (about 64 KB) -- one 4-double
// partial sum per block for at most kNoAllocMaxBlocks blocks, then an arrival counter.  Every GPU
// that loads this library holds it until the process exits.  A call accepts at most
// kNoAllocMaxBeads (4,194,304) beads and returns SOUFFLE_ERR_BAD_INPUT beyond that.  All calls
// share the one array, and each call leaves its partial sums in it; the arrival counter, the only
// part that must start at zero, is cleared at the start of every call.  Calls that overlap on the
// GPU (on different streams, or from host threads without ordering between them) race on the
// array and give wrong results: order them on one stream.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "souffle_gpu.h"

namespace souffle {
void record_error(const std::string& msg);  // souffle_gpu.cu: text for souffle_gpu_last_error()
}

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 2048;
constexpr int kNoAllocBeadsPerThread = 8;
constexpr long long kNoAllocMaxBeads =
    (long long)kNoAllocMaxBlocks * kNoAllocThreads * kNoAllocBeadsPerThread;  // 4,194,304
constexpr int kNoAllocCounter = 4 * kNoAllocMaxBlocks;                         // index of the counter
constexpr int kNoAllocScratchDoubles = 4 * kNoAllocMaxBlocks + 32;

// The scratch.  In host code this name is only a stand-in for the device array; the device
// address is obtained with cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// KE = sum 1/2 m |v|^2 (particle_kinetic_energy, src/energies.cpp:13-22) and the plain velocity
// sum (what the COM removal of src/md.cpp:505-514 divides by N).  Each thread takes a fixed set
// of beads, blocks reduce with a fixed tree, and the last block to arrive adds the block sums in
// block order, so the result is the same on every call.
__global__ void __launch_bounds__(kNoAllocThreads) k_kinetic_noalloc(const double* vel, const double* mass,
                                                                      long long n, double* scr, double* out) {
  __shared__ double red[kNoAllocThreads / 32][4];
  __shared__ bool last;
  unsigned int* arrivals = reinterpret_cast<unsigned int*>(scr + kNoAllocCounter);
  double k = 0, x = 0, y = 0, z = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    const double m = mass ? mass[i] : 1.0;
    k += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    x += vx;
    y += vy;
    z += vz;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    k += __shfl_xor_sync(0xffffffffu, k, o);
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
    z += __shfl_xor_sync(0xffffffffu, z, o);
  }
  if (lane == 0) {
    red[wid][0] = k;
    red[wid][1] = x;
    red[wid][2] = y;
    red[wid][3] = z;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[4] = {0, 0, 0, 0};
    for (int w = 0; w < kNoAllocThreads / 32; w++)
      for (int c = 0; c < 4; c++) s[c] += red[w][c];
    for (int c = 0; c < 4; c++) scr[4 * blockIdx.x + c] = s[c];
    __threadfence();
    last = (atomicAdd(arrivals, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double s[4] = {0, 0, 0, 0};
  for (unsigned int b = 0; b < gridDim.x; b++)
    for (int c = 0; c < 4; c++) s[c] += __ldcg(&scr[4 * b + c]);
  for (int c = 0; c < 4; c++) out[c] = s[c];
  *arrivals = 0;
}

souffle_status noalloc_fail(souffle_status s, const std::string& msg) {
  souffle::record_error("souffle_gpu_kinetic_energy_noalloc: " + msg);
  return s;
}

}  // namespace

extern "C" souffle_status souffle_gpu_kinetic_energy_noalloc(const double* vel, const double* mass,
                                                             int64_t n_beads, double* out, void* stream) {
  if (!vel || !out || n_beads < 0) return noalloc_fail(SOUFFLE_ERR_BAD_INPUT, "null pointer or negative count");
  if (n_beads > kNoAllocMaxBeads)
    return noalloc_fail(SOUFFLE_ERR_BAD_INPUT, std::to_string((long long)n_beads) +
                                                   " beads exceed the fixed scratch limit of " +
                                                   std::to_string(kNoAllocMaxBeads));
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return noalloc_fail(SOUFFLE_ERR_NO_DEVICE, "no current CUDA device");
  double* scr;
  {
    // set-up, once per device with that device current: the scratch array's device address
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return noalloc_fail(SOUFFLE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scr = g_scratch_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(scr + kNoAllocCounter, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) {
    if (n_beads == 0) {
      e = cudaMemsetAsync(out, 0, 4 * sizeof(double), s);
    } else {
      long long blocks = (n_beads + kNoAllocThreads - 1) / kNoAllocThreads;
      if (blocks > kNoAllocMaxBlocks) blocks = kNoAllocMaxBlocks;
      k_kinetic_noalloc<<<(unsigned)blocks, kNoAllocThreads, 0, s>>>(vel, mass, n_beads, scr, out);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) return noalloc_fail(SOUFFLE_ERR_CUDA, cudaGetErrorString(e));
  return SOUFFLE_OK;
}
