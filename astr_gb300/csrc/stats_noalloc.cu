// Kinetic-energy / enstrophy reduction that allocates nothing.
//
// Some callers of this library cannot call cudaMalloc: a host that hands
// every byte of HBM to its own memory pool or to the serving loop's
// admission-by-free-memory, or a time loop that must not let an allocation
// (which may synchronise the device) happen between steps.  This entry point
// computes the same statistics as astr_gpu_reduce_stats from device arrays
// the caller already owns, with its per-block partial sums in a file-scope
// device array instead of context memory.
#include "../../include/astr_gpu.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kHM = 5;
constexpr int kThreads = 256;
constexpr int kPointsPerThread = 16;
constexpr long long kPointsPerBlock = (long long)kThreads * kPointsPerThread;

// Two partial sums per block; every GPU that loads the library holds this
// array (1 MiB) until the process exits.
static __device__ __align__(256) double g_stats_scratch[2 * ASTR_NOALLOC_STATS_MAX_BLOCKS];

struct Dims {
  int im, jm, km, ndims;
  long long NI, NJ, I, J, n0;
};

__global__ void k_stats_partials(Dims g, const double* __restrict__ rho,
                                 const double* __restrict__ vel,
                                 const double* __restrict__ dvel, double* part) {
  const long long nh = g.NI * g.NJ * (long long)(g.km + 2 * kHM + 1);
  double ke = 0.0, en = 0.0;
  const long long base = (long long)blockIdx.x * kPointsPerBlock;
  for (int r = 0; r < kPointsPerThread; ++r) {
    const long long idx = base + (long long)r * kThreads + threadIdx.x;
    if (idx >= g.n0) break;
    const int i = (int)(idx % g.I);
    const long long t = idx / g.I;
    const int j = (int)(t % g.J);
    const int k = (int)(t / g.J);
    const bool ink = g.ndims == 3 ? (k >= 1) : (k == 0);
    if (i < 1 || j < 1 || !ink) continue;
    const long long p = (long long)(i + kHM) + g.NI * ((long long)(j + kHM) + g.NJ * (long long)(k + kHM));
    const double ro = rho[p], u = vel[p], v = vel[p + nh], w = vel[p + 2 * nh];
    ke += ro * (u * u + v * v + w * w);
    const double* G = dvel + idx;
    const long long n0 = g.n0;
    const double o3 = G[1 * n0] - G[3 * n0];
    double om = o3 * o3;
    if (g.ndims == 3) {
      const double o1 = G[5 * n0] - G[7 * n0];
      const double o2 = G[6 * n0] - G[2 * n0];
      om = o1 * o1 + o2 * o2 + o3 * o3;
    }
    en += ro * om;
  }
  __shared__ double sk[kThreads], se[kThreads];
  sk[threadIdx.x] = ke;
  se[threadIdx.x] = en;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sk[threadIdx.x] += sk[threadIdx.x + s];
      se[threadIdx.x] += se[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sk[0];
    part[2 * blockIdx.x + 1] = se[0];
  }
}

// Sums the nblocks partials in a fixed order into out2.  Every partial read
// here was written by k_stats_partials in the same call, so the scratch
// needs no clearing; whatever an earlier call left there is never read.
__global__ void k_stats_total(double* part, int nblocks, double* out2) {
  __shared__ double sk[1024], se[1024];
  double ke = 0.0, en = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    ke += part[2 * b];
    en += part[2 * b + 1];
  }
  sk[threadIdx.x] = ke;
  se[threadIdx.x] = en;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sk[threadIdx.x] += sk[threadIdx.x + s];
      se[threadIdx.x] += se[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out2[0] = sk[0];
    out2[1] = se[0];
  }
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array in the current context.  The array's
// name is only a host-side stand-in in host code, so its address is looked
// up with cudaGetSymbolAddress on every call whose stream is not being
// captured (the lookup follows the current context, so a cudaDeviceReset or
// another context on the same device never leaves a stale address behind).
// While a capture is active the address recorded by the last uncaptured call
// on this device is used; with none recorded the call fails.
int scratch_for_current_device(cudaStream_t st, double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ASTR_ERR_CUDA;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const bool capturing = cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!capturing) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_stats_scratch) != cudaSuccess || !p) return ASTR_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  if (!g_scratch_ptr[dev]) return ASTR_ERR_CUDA;
  *out = g_scratch_ptr[dev];
  return ASTR_OK;
}

}  // namespace

extern "C" int astr_gpu_stats_noalloc(const double* rho, const double* vel, const double* dvel,
                                      const astr_dims* dims, double l0, void* stream,
                                      double* kenergy, double* enstrophy) {
  if (!rho || !vel || !dvel || !dims || !kenergy || !enstrophy) return ASTR_ERR_ARG;
  Dims g;
  g.im = dims->im; g.jm = dims->jm; g.km = dims->km;
  g.ndims = dims->ka > 0 ? 3 : 2;
  // the block sizes astr_gpu_create accepts: im, jm (, km) >= 8, km == 0 in 2-D
  if (g.im < 8 || g.jm < 8 || (g.ndims == 3 && g.km < 8) || (g.ndims == 2 && g.km != 0))
    return ASTR_ERR_ARG;
  g.NI = g.im + 2 * kHM + 1;
  g.NJ = g.jm + 2 * kHM + 1;
  g.I = g.im + 1;
  g.J = g.jm + 1;
  g.n0 = g.I * g.J * (long long)(g.km + 1);
  const long long nblocks = (g.n0 + kPointsPerBlock - 1) / kPointsPerBlock;
  // one slot pair per block plus the result pair must fit the scratch array
  if (nblocks + 1 > ASTR_NOALLOC_STATS_MAX_BLOCKS) return ASTR_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* scratch = nullptr;
  const int rc = scratch_for_current_device(st, &scratch);
  if (rc != ASTR_OK) return rc;
  // cudaLaunchKernel returns each launch's own status, so an error left
  // pending by the caller's unrelated work is neither reported here nor
  // cleared
  {
    void* args[] = {&g, (void*)&rho, (void*)&vel, (void*)&dvel, &scratch};
    if (cudaLaunchKernel((const void*)k_stats_partials, dim3((unsigned)nblocks), dim3(kThreads), args,
                         0, st) != cudaSuccess)
      return ASTR_ERR_CUDA;
  }
  double* result = scratch + 2 * nblocks;
  {
    int nb = (int)nblocks;
    void* args[] = {&scratch, &nb, &result};
    if (cudaLaunchKernel((const void*)k_stats_total, dim3(1), dim3(1024), args, 0, st) != cudaSuccess)
      return ASTR_ERR_CUDA;
  }
  double h[2];
  if (cudaMemcpyAsync(h, result, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return ASTR_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return ASTR_ERR_CUDA;
  const double npts = g.ndims == 3 ? (double)dims->ia * dims->ja * dims->ka
                                   : (double)dims->ia * dims->ja;
  const double roinf = 1.0, uinf = 1.0, len = l0 > 0.0 ? l0 : 1.0;
  *kenergy = 0.5 * h[0] / npts / (roinf * uinf * uinf);
  *enstrophy = 0.5 * h[1] / npts / (roinf * ((uinf / len) * (uinf / len)));
  return ASTR_OK;
}
