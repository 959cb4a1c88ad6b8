// chf_static.cu -- the allocation-free statistics entry point.
//
// Some callers cannot allocate device memory: a host model whose device memory
// is owned by another runtime (a coupler or framework that preallocates one
// pool and forbids further cudaMalloc), a run that has committed the device's
// memory to the resident state, or a time loop that must not pay the
// synchronisation and latency of cudaMalloc/cudaFree.  chf_diagnostics_static
// gives them the energy diagnostics of chf_diagnostics on their own device
// arrays without any allocation: it needs no handle, and the reduction's
// scratch -- the per-plane partial sums a first kernel writes and a second
// kernel reads -- lives in a file-scope __device__ array of fixed size.
//
// Limits and sharing: at most CHF_STATIC_MAX_PLANES wall-normal planes
// (nnz + 1 <= 1025); larger grids, and grids that chf_create would reject
// (nnx or nny not a multiple of 4, nnz odd or below 4), are rejected with
// CHF_E_INVALID before any CUDA call.  The call waits for its stream and
// returns its results in host memory.  Every
// device that loads the library holds the array (about 33 KB) until the
// process exits.  All calls share it: every slot is written before it is
// read within one call, so nothing has to be cleared between calls, and the
// array keeps the last call's values; calls that overlap on the GPU (two
// streams, or two host threads) race on it and must be serialised by the
// caller.  The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current and caches it; later calls
// on that device reuse it.  Make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/chflow.h"

namespace {

constexpr int MAX_PLANES = CHF_STATIC_MAX_PLANES;
constexpr int SLOT = 4;  // per plane: energy, max |value|, non-finite count, spare

// [MAX_PLANES] plane partials + 1 slot of totals
static __device__ __align__(256) double g_stat_scratch[(MAX_PLANES + 1) * SLOT];

// One CTA per wall-normal plane k: the spectral energy
// 0.5 * sum (u^2 + v^2 + w^2) over the plane without the spanwise Nyquist
// slot, the largest |value| of the six fields and the count of non-finite
// values, written to slot k of the scratch.
__global__ void k_stat_planes(const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, const double* __restrict__ ox,
                              const double* __restrict__ oy, const double* __restrict__ oz,
                              long plane, int nnx, int nyq, double* scratch) {
  const int k = blockIdx.x;
  const size_t base = (size_t)k * plane;
  double e = 0.0, mx = 0.0, bad = 0.0;
  for (long i = threadIdx.x; i < plane; i += blockDim.x) {
    if (i / nnx == nyq) continue;  // (x index, y index) = (i % nnx, i / nnx)
    const size_t j = base + i;
    const double a = u[j], b = v[j], c = w[j];
    e += 0.5 * (a * a) + 0.5 * (b * b) + 0.5 * (c * c);
    const double vals[6] = {a, b, c, ox[j], oy[j], oz[j]};
    for (int q = 0; q < 6; ++q) {
      if (!isfinite(vals[q])) bad += 1.0;
      else mx = fmax(mx, fabs(vals[q]));
    }
  }
  __shared__ double se[32], sm[32], sb[32];
  for (int off = 16; off > 0; off >>= 1) {
    e += __shfl_down_sync(0xffffffffu, e, off);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
    bad += __shfl_down_sync(0xffffffffu, bad, off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    se[warp] = e;
    sm[warp] = mx;
    sb[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double te = 0.0, tm = 0.0, tb = 0.0;
    for (int q = 0; q < nw; ++q) {
      te += se[q];
      tm = fmax(tm, sm[q]);
      tb += sb[q];
    }
    scratch[(size_t)k * SLOT + 0] = te;
    scratch[(size_t)k * SLOT + 1] = tm;
    scratch[(size_t)k * SLOT + 2] = tb;
    scratch[(size_t)k * SLOT + 3] = 0.0;
  }
}

// Totals over the nplanes partials, in plane order (deterministic), into the
// last slot.
__global__ void k_stat_total(int nplanes, double* scratch) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double te = 0.0, tm = 0.0, tb = 0.0;
  for (int k = 0; k < nplanes; ++k) {
    te += scratch[(size_t)k * SLOT + 0];
    tm = fmax(tm, scratch[(size_t)k * SLOT + 1]);
    tb += scratch[(size_t)k * SLOT + 2];
  }
  double* t = scratch + (size_t)MAX_PLANES * SLOT;
  t[0] = te;
  t[1] = tm;
  t[2] = tb;
  t[3] = (double)nplanes;
}

std::mutex g_mu;
double* g_ptr[64] = {};  // device address of g_stat_scratch per device ordinal

}  // namespace

extern "C" int chf_diagnostics_static(int nnx, int nny, int nnz, const double* d_unp1,
                                      const double* d_vnp1, const double* d_wnp1,
                                      const double* d_omegaxnp1, const double* d_omegaynp1,
                                      const double* d_omegaznp1, double* energy_profile,
                                      chf_diag* out, void* stream) {
  // the grid rules of chf_create: (re, im) pairs along x and a spanwise
  // Nyquist slot at nny / 2 need nnx and nny to be multiples of 4
  if (nnx < 4 || nnx % 4 || nny < 4 || nny % 4 || nnz < 4 || nnz % 2 || !d_unp1 || !d_vnp1 || !d_wnp1 ||
      !d_omegaxnp1 || !d_omegaynp1 || !d_omegaznp1 || !out)
    return CHF_E_INVALID;
  if (nnz + 1 > MAX_PLANES) return CHF_E_INVALID;  // the fixed scratch holds 1025 planes
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CHF_E_CUDA;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ptr[dev]) {
      // first call on this device: the array's device address, looked up
      // with the device current
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_stat_scratch) != cudaSuccess || !p) return CHF_E_CUDA;
      g_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nplanes = nnz + 1;
  const long plane = (long)nnx * nny;
  k_stat_planes<<<nplanes, 256, 0, st>>>(d_unp1, d_vnp1, d_wnp1, d_omegaxnp1, d_omegaynp1,
                                         d_omegaznp1, plane, nnx, nny / 2, scratch);
  k_stat_total<<<1, 32, 0, st>>>(nplanes, scratch);
  if (cudaGetLastError() != cudaSuccess) return CHF_E_CUDA;
  double tot[4];
  if (cudaMemcpyAsync(tot, scratch + (size_t)MAX_PLANES * SLOT, sizeof(tot), cudaMemcpyDeviceToHost,
                      st) != cudaSuccess)
    return CHF_E_CUDA;
  if (energy_profile &&
      cudaMemcpy2DAsync(energy_profile, sizeof(double), scratch, SLOT * sizeof(double), sizeof(double),
                        nplanes, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return CHF_E_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return CHF_E_CUDA;
  out->energy = tot[0];
  out->max_abs = tot[1];
  out->finite = tot[2] == 0.0 ? 1 : 0;
  out->wall_shear_top = 0.0;     // needs au0, which this entry point does not take
  out->wall_shear_bottom = 0.0;
  return out->finite ? CHF_OK : CHF_E_NUMERIC;
}
