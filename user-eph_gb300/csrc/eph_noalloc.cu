// Electronic-grid solve that allocates nothing (eph_fdm_solve_noalloc in
// include/eph_gb.h).
//
// Who needs it: callers that own every byte of device memory themselves and
// may not call cudaMalloc/cudaFree during a run -- an MD engine that sizes one
// device pool at start-up and hands out slices of it, or a time-step loop
// that must not synchronise the device (cudaMalloc and cudaFree can).  The
// caller passes every input and output as device pointers; the only other
// memory used is the file-scope array below, reserved when the library is
// loaded and held on every GPU that loads it until the process exits.
//
// Shared scratch: every call uses the same array and leaves the last call's
// contents in it.  Calls whose work overlaps on the GPU (two streams, or two
// threads issuing on different streams) race on it; order them on one stream
// or serialise them.  Nothing in the array has to start at zero: the
// reduction slots and the ping-pong grid are fully written before they are
// read.
#include <atomic>
#include <cmath>
#include <cstdint>

#include <cuda_runtime.h>

#include "eph_gb.h"

namespace {

constexpr int kMaxDevices = 64;

// [0, MAX_CELLS): second temperature buffer; [MAX_CELLS, +3): c_min, rho_min,
// kappa_max of the stability rule.
static __device__ __align__(256) double g_fdm_scratch[EPH_NOALLOC_MAX_CELLS + 8];

// Device address of g_fdm_scratch per device, filled on the first call on
// that device (host code cannot use the symbol itself as an address).  Two
// host threads making their first call on one device at once both look the
// address up and store the same value.
std::atomic<double *> g_scratch_addr[kMaxDevices];

__global__ void k_noalloc_bounds(long ntotal, const double *__restrict__ C, const double *__restrict__ rho,
                                 const double *__restrict__ kappa, const signed char *__restrict__ flag,
                                 double *__restrict__ out) {
  // eph_fdm.h:290-300: start from cell 0 whatever its flag, then every cell
  // that is not CONSTANT_VALUE
  double c_min = C[0], r_min = rho[0], k_max = kappa[0];
  for (long i = 1 + threadIdx.x; i < ntotal; i += blockDim.x)
    if (flag[i] != 0) {
      c_min = fmin(c_min, C[i]);
      r_min = fmin(r_min, rho[i]);
      k_max = fmax(k_max, kappa[i]);
    }
  __shared__ double s[3][256];
  s[0][threadIdx.x] = c_min;
  s[1][threadIdx.x] = r_min;
  s[2][threadIdx.x] = k_max;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + h]);
      s[1][threadIdx.x] = fmin(s[1][threadIdx.x], s[1][threadIdx.x + h]);
      s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s[0][0];
    out[1] = s[1][0];
    out[2] = s[2][0];
  }
}

// One substep of EPH_FDM::solve (eph_fdm.h:315-396), the reference's
// expression order: T_out from T_in.
__global__ void k_noalloc_substep(long nx, long ny, long nz, double dx, double dy, double dz, double inner_dt,
                                  const double *__restrict__ T, double *__restrict__ Tout,
                                  const double *__restrict__ kappa, const double *__restrict__ rho,
                                  const double *__restrict__ C, const double *__restrict__ S,
                                  const double *__restrict__ dT, const signed char *__restrict__ flag) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long ntotal = nx * ny * nz;
  if (r >= ntotal) return;
  const long i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
  double ddT = 0.0;
  if (flag[r] != 2) {
    long p, q;
    p = (i > 0) ? r - 1 : r + (nx - 1);
    q = (i < nx - 1) ? r + 1 : r - (nx - 1);
    if (flag[q] == 2) q = r;
    else if (flag[p] == 2) p = r;
    ddT += (kappa[q] - kappa[p]) * (T[q] - T[p]) / dx / dx / 4.0;
    ddT += kappa[r] * ((T[q] + T[p] - 2.0 * T[r]) / dx / dx);
    p = (j > 0) ? r - nx : r + (ny - 1) * nx;
    q = (j < ny - 1) ? r + nx : r - (ny - 1) * nx;
    if (flag[q] == 2) q = r;
    else if (flag[p] == 2) p = r;
    ddT += (kappa[q] - kappa[p]) * (T[q] - T[p]) / dy / dy / 4.0;
    ddT += kappa[r] * ((T[q] + T[p] - 2.0 * T[r]) / dy / dy);
    p = (k > 0) ? r - nx * ny : r + (nz - 1) * nx * ny;
    q = (k < nz - 1) ? r + nx * ny : r - (nz - 1) * nx * ny;
    if (flag[q] == 2) q = r;
    else if (flag[p] == 2) p = r;
    ddT += (kappa[q] - kappa[p]) * (T[q] - T[p]) / dz / dz / 4.0;
    ddT += kappa[r] * ((T[q] + T[p] - 2.0 * T[r]) / dz / dz);
  }
  double t = T[r];
  if (flag[r] == 1) t += (ddT + dT[r] + S[r]) / (rho[r] * C[r]) * inner_dt;
  if (t < 0.0) t = 0.0;
  Tout[r] = t;
}

}  // namespace

extern "C" int eph_fdm_solve_noalloc(long nx, long ny, long nz, const double *lo, const double *hi, double dt,
                                     long steps, double *T, const double *dT, const double *S, const double *rho_e,
                                     const double *C_e, const double *kappa, const signed char *flag, void *stream,
                                     unsigned *nsub_out) {
  if (nx < 1 || ny < 1 || nz < 1 || !lo || !hi || !(dt > 0) || steps < 1 || !T || !dT || !S || !rho_e || !C_e ||
      !kappa || !flag)
    return EPH_ERR_ARG;
  const long ntotal = nx * ny * nz;
  if (ntotal > EPH_NOALLOC_MAX_CELLS) return EPH_ERR_CAPACITY;  // larger than the static scratch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return EPH_ERR_CUDA;
  double *scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    // set-up, once per device, with that device current
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_fdm_scratch) != cudaSuccess || !p) return EPH_ERR_CUDA;
    scratch = static_cast<double *>(p);
    g_scratch_addr[dev].store(scratch, std::memory_order_release);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // grid spacing as eph_fdm.h:127-146 computes it
  const double dx = (hi[0] - lo[0]) / (double)(size_t)nx;
  const double dy = (hi[1] - lo[1]) / (double)(size_t)ny;
  const double dz = (hi[2] - lo[2]) / (double)(size_t)nz;
  // stability substeps, eph_fdm.h:275-313
  k_noalloc_bounds<<<1, 256, 0, st>>>(ntotal, C_e, rho_e, kappa, flag, scratch + EPH_NOALLOC_MAX_CELLS);
  double b[3];
  if (cudaMemcpyAsync(b, scratch + EPH_NOALLOC_MAX_CELLS, sizeof b, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return EPH_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return EPH_ERR_CUDA;
  // the reference only asserts positive bounds; here a zero or negative C_e
  // or rho_e (cell 0 enters the minimum whatever its flag) is an argument
  // error, and so is a substep count above EPH_NOALLOC_MAX_SUBSTEPS, before
  // anything is launched
  if (!(b[0] > 0.0) || !(b[1] > 0.0) || !(b[2] >= 0.0)) return EPH_ERR_ARG;
  if (steps > EPH_NOALLOC_MAX_SUBSTEPS) return EPH_ERR_ARG;
  double inner_dt = dt / (double)(size_t)steps;
  const double dtdxdydz = inner_dt * (1.0 / dx / dx + 1.0 / dy / dy + 1.0 / dz / dz);
  const double r = dtdxdydz / b[0] / b[1] * b[2];
  unsigned nsub = (unsigned)steps;
  if (r > 0.4) {
    inner_dt = 0.4 * inner_dt / r;
    const double want = dt / inner_dt;
    if (!(want < (double)EPH_NOALLOC_MAX_SUBSTEPS + 1.0)) return EPH_ERR_ARG;
    const unsigned s = (unsigned)want;
    nsub = s > 1u ? s : 1u;
    inner_dt = dt / nsub;
  }
  const int threads = 64;
  const int blocks = (int)((ntotal + threads - 1) / threads);
  double *src = T, *dst = scratch;
  for (unsigned s = 0; s < nsub; ++s) {
    k_noalloc_substep<<<blocks, threads, 0, st>>>(nx, ny, nz, dx, dy, dz, inner_dt, src, dst, kappa, rho_e, C_e, S,
                                                  dT, flag);
    double *t = src;
    src = dst;
    dst = t;
  }
  if (src != T && cudaMemcpyAsync(T, src, sizeof(double) * (size_t)ntotal, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return EPH_ERR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return EPH_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return EPH_ERR_CUDA;
  if (nsub_out) *nsub_out = nsub;
  return EPH_OK;
}
