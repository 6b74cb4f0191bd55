// Element-level testing entry points: evaluate the device beam and contact
// elements on caller-supplied packed states, so the kernels can be compared
// with a CPU evaluation of compute_beams / compute_contact_beams for the
// same inputs.
//
// Packed input record (96 doubles): X1[3] X2[3] u1[3] u2[3] R1[9] R2[9] ΔR1[9]
// ΔR2[9] u̇1[3] u̇2[3] ẇ1[3] ẇ2[3] ü1[3] ü2[3] ẅ1[3] ẅ2[3] l0 Rₑ⁰[9] K̄ū K̄Θ[3]
// K̄ΘΘ[3] Jᵨ[3] Aᵨ damping radius (pad).  3x3 matrices column-major.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/endobeams_gb300.h"
#include "eb_contact.cuh"

using namespace ebd;

namespace {
thread_local char g_err2[512];

__device__ __forceinline__ V3 P3(const double* p) { return v3(p[0], p[1], p[2]); }
__device__ __forceinline__ M3 P9(const double* p) {
  M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = p[k];
  return m;
}

__global__ void k_element_eval(int64_t n, const double* in, Gauss3 g, double* out) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double* p = in + 96 * e;
  double* o = out + 458 * e;
  BeamIn b;
  b.X1 = P3(p + 0); b.X2 = P3(p + 3); b.u1 = P3(p + 6); b.u2 = P3(p + 9);
  b.R1 = P9(p + 12); b.R2 = P9(p + 21); b.dR1 = P9(p + 30); b.dR2 = P9(p + 39);
  b.ud1 = P3(p + 48); b.ud2 = P3(p + 51); b.wd1 = P3(p + 54); b.wd2 = P3(p + 57);
  b.udd1 = P3(p + 60); b.udd2 = P3(p + 63); b.wdd1 = P3(p + 66); b.wdd2 = P3(p + 69);
  b.l0 = p[72]; b.Re0 = P9(p + 73); b.Ku = p[82]; b.KT = P3(p + 83); b.KTT = P3(p + 86); b.Jr = P3(p + 89);
  b.Ar = p[92]; b.damping = p[93];
  BeamOut bo{o + 26, o + 170, o + 314, o + 2, o + 14, o + 0};
  beam_element(b, g, bo);
}

__global__ void k_contact_eval(int64_t n, const double* in, Gauss3 g, ContactProps cp, SurfaceDev s, double* out,
                               int32_t* flags) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double* p = in + 96 * e;
  double* o = out + 301 * e;
  ContactIn c;
  c.X1 = P3(p + 0); c.X2 = P3(p + 3); c.u1 = P3(p + 6); c.u2 = P3(p + 9);
  c.R1 = P9(p + 12); c.R2 = P9(p + 21); c.dR1 = P9(p + 30); c.dR2 = P9(p + 39);
  c.ud1 = P3(p + 48); c.ud2 = P3(p + 51); c.wd1 = P3(p + 54); c.wd2 = P3(p + 57);
  c.l0 = p[72]; c.Re0 = P9(p + 73); c.radius = p[94];
  ContactOut co{o + 13, o + 157, o + 1, o + 0};
  bool any = false;
  contact_element(c, g, cp, s, co, &any);
  flags[e] = any ? 1 : 0;
}

struct DBuf {
  void* p = nullptr;
  ~DBuf() { if (p) cudaFree(p); }
};

}  // namespace

// defined in eb_abi.cu
std::vector<double> eb_sdf_coefficients_host(const double* values, const int64_t dims[3], bool negate);
std::vector<double> eb_sdf_samples_padded_host(const double* values, const int64_t dims[3], bool negate);
int eb_internal_fail(int code, const char* msg);

namespace {
int err(const char* what, cudaError_t e) {
  std::snprintf(g_err2, sizeof(g_err2), "%s: %s", what, cudaGetErrorString(e));
  return eb_internal_fail(EB_ERR_CUDA, g_err2);
}
}  // namespace

extern "C" int eb_element_eval(int64_t n, const double* in, const double* gauss6, double* out) {
  if (n <= 0 || !in || !gauss6 || !out) return EB_ERR_ARG;
  Gauss3 g;
  for (int i = 0; i < 3; ++i) { g.w[i] = gauss6[i]; g.z[i] = gauss6[3 + i]; }
  DBuf di, dout;
  cudaError_t e;
  if ((e = cudaMalloc(&di.p, sizeof(double) * 96 * n)) != cudaSuccess) return err("cudaMalloc", e);
  if ((e = cudaMalloc(&dout.p, sizeof(double) * 458 * n)) != cudaSuccess) return err("cudaMalloc", e);
  cudaMemcpy(di.p, in, sizeof(double) * 96 * n, cudaMemcpyHostToDevice);
  cudaMemset(dout.p, 0, sizeof(double) * 458 * n);
  k_element_eval<<<(unsigned)((n + 127) / 128), 128>>>(n, (const double*)di.p, g, (double*)dout.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return err("k_element_eval launch", e);
  if ((e = cudaMemcpy(out, dout.p, sizeof(double) * 458 * n, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return err("k_element_eval", e);
  return EB_OK;
}

extern "C" int eb_contact_eval(int64_t n, const double* in, const double* gauss6, const double* props,
                               const double* surf, const double* values, double* out, int32_t* flags) {
  if (n <= 0 || !in || !gauss6 || !props || !surf || !out || !flags) return EB_ERR_ARG;
  Gauss3 g;
  for (int i = 0; i < 3; ++i) { g.w[i] = gauss6[i]; g.z[i] = gauss6[3 + i]; }
  ContactProps cp{props[0], props[1], props[2], props[3]};
  SurfaceDev s;
  std::memset(&s, 0, sizeof(s));
  s.kind = (int)surf[0];
  s.cx = surf[1]; s.cy = surf[2]; s.cz = surf[3]; s.R = surf[4];
  if (s.kind == 2) {
    s.axis = (int)surf[1];
    s.pos = surf[2];
  }
  if (s.kind < 0 || s.kind > 3 || s.axis < 0 || s.axis > 2) return EB_ERR_ARG;
  if (s.kind == 3) {  // voxel SDF, trilinear
    s.kind = 1;
    s.interp = 1;
    if (surf[5] < 2 || surf[6] < 2 || surf[7] < 2) return EB_ERR_ARG;
  }
  DBuf dcoef, di, dout, dfl;
  cudaError_t e;
  if (s.kind == 1) {
    if (!values) return EB_ERR_ARG;
    int64_t dims[3] = {(int64_t)surf[5], (int64_t)surf[6], (int64_t)surf[7]};
    std::vector<double> c = s.interp ? eb_sdf_samples_padded_host(values, dims, false)
                                     : eb_sdf_coefficients_host(values, dims, false);
    if ((e = cudaMalloc(&dcoef.p, sizeof(double) * c.size())) != cudaSuccess) return err("cudaMalloc", e);
    cudaMemcpy(dcoef.p, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice);
    s.coef = (const double*)dcoef.p;
    s.nx = (int)dims[0]; s.ny = (int)dims[1]; s.nz = (int)dims[2];
    s.x0 = surf[8]; s.y0 = surf[9]; s.z0 = surf[10];
    s.ihx = 1.0 / surf[11]; s.ihy = 1.0 / surf[12]; s.ihz = 1.0 / surf[13];
    s.xl = (s.nx - 1) * surf[11]; s.yl = (s.ny - 1) * surf[12]; s.zl = (s.nz - 1) * surf[13];
  }
  if ((e = cudaMalloc(&di.p, sizeof(double) * 96 * n)) != cudaSuccess) return err("cudaMalloc", e);
  if ((e = cudaMalloc(&dout.p, sizeof(double) * 301 * n)) != cudaSuccess) return err("cudaMalloc", e);
  if ((e = cudaMalloc(&dfl.p, sizeof(int32_t) * n)) != cudaSuccess) return err("cudaMalloc", e);
  cudaMemcpy(di.p, in, sizeof(double) * 96 * n, cudaMemcpyHostToDevice);
  cudaMemset(dout.p, 0, sizeof(double) * 301 * n);
  k_contact_eval<<<(unsigned)((n + 127) / 128), 128>>>(n, (const double*)di.p, g, cp, s, (double*)dout.p,
                                                      (int32_t*)dfl.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return err("k_contact_eval launch", e);
  if ((e = cudaMemcpy(out, dout.p, sizeof(double) * 301 * n, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return err("k_contact_eval", e);
  cudaMemcpy(flags, dfl.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  return EB_OK;
}

// ---------------------------------------------------------------- contact evaluation without allocation
// Variant of eb_contact_eval for callers that cannot allocate device memory
// during the call (a host whose device memory belongs to its own pool
// allocator, a loop that forbids allocation after start-up): the caller's
// device buffers are used directly, and the prefiltered SDF coefficients go
// to the fixed array below instead of a cudaMalloc.
namespace {

__device__ __align__(256) double g_noalloc_coef[EB_NOALLOC_SDF_MAX_COEFS];

std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
// Device address of g_noalloc_coef per device ordinal, and the context it was looked up in:
// after cudaDeviceReset (or any other re-creation of the device's context) the address is
// looked up again.
double* g_noalloc_ptr[kMaxDevices] = {nullptr};
void* g_noalloc_ctx[kMaxDevices] = {nullptr};

// The calling thread's current driver context (an opaque handle), through the runtime's
// driver entry-point query so the library does not link the driver API; nullptr if unknown.
void* current_context() {
  using GetCurrent = int (*)(void**);
  static GetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (GetCurrent)f;
  }();
  void* ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

__global__ void k_sdf_interior(const double* __restrict__ vals, int nx, int ny, int nz, double* __restrict__ c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nx * ny * nz) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((int64_t)nx * ny));
  c[(i + 1) + (int64_t)(nx + 2) * ((j + 1) + (int64_t)(ny + 2) * (k + 1))] = vals[t];
}

// One thread per grid line along `axis`: in-place solve of the quadratic
// B-spline interpolation system ⅛c[i-1] + ¾c[i] + ⅛c[i+1] = y[i] with the
// reflected ends (first/last diagonal 7/8), then the two pads c[0] = c[1],
// c[n+1] = c[n].  Lines run over the padded range of axes already filtered.
__global__ void k_sdf_prefilter_axis(double* c, int nx, int ny, int nz, int axis) {
  const int64_t px = nx + 2, py = ny + 2;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int n;
  int64_t base, stride;
  if (axis == 0) {  // lines (j, k), interior j and k
    if (t >= (int64_t)ny * nz) return;
    const int64_t j = 1 + t % ny, k = 1 + t / ny;
    n = nx; stride = 1; base = px * (j + py * k);
  } else if (axis == 1) {  // lines (i, k), all i, interior k
    if (t >= px * nz) return;
    const int64_t i = t % px, k = 1 + t / px;
    n = ny; stride = px; base = i + px * py * k;
  } else {  // lines (i, j), all i and j
    if (t >= px * py) return;
    const int64_t i = t % px, j = t / px;
    n = nz; stride = px * py; base = i + px * j;
  }
  double* y = c + base + stride;  // first interior point of the line
  if (n > 1) {
    double cpa[32];
    double cp = 0.125 / 0.875;
    cpa[0] = cp;
    y[0] = y[0] / 0.875;
    for (int i = 1; i < n; ++i) {
      const bool last = i == n - 1;
      const double m = (last ? 0.875 : 0.75) - 0.125 * cp;
      y[i * stride] = (y[i * stride] - 0.125 * y[(i - 1) * stride]) / m;
      cp = last ? 0.0 : 0.125 / m;
      if (i < 32) cpa[i] = cp;
    }
    // beyond the first 32 rows the factor has converged to its fixed point
    for (int i = n - 2; i >= 0; --i) y[i * stride] -= cpa[i < 32 ? i : 31] * y[(i + 1) * stride];
  }
  y[-stride] = y[0];
  y[n * stride] = y[(n - 1) * stride];
}

}  // namespace

// Prefilters a padded coefficient grid whose interior holds the SDF samples
// (three passes, one thread per grid line).
namespace eb {
void launch_sdf_prefilter(double* coef, int nx, int ny, int nz, cudaStream_t st) {
  const int64_t px = nx + 2, py = ny + 2;
  k_sdf_prefilter_axis<<<(unsigned)(((int64_t)ny * nz + 127) / 128), 128, 0, st>>>(coef, nx, ny, nz, 0);
  k_sdf_prefilter_axis<<<(unsigned)((px * nz + 127) / 128), 128, 0, st>>>(coef, nx, ny, nz, 1);
  k_sdf_prefilter_axis<<<(unsigned)((px * py + 127) / 128), 128, 0, st>>>(coef, nx, ny, nz, 2);
}
}  // namespace eb

extern "C" int eb_contact_eval_noalloc(int64_t n, const double* d_in, const double* gauss6, const double* props,
                                       const double* surf, const double* d_sdf_values, double* d_out,
                                       int32_t* d_flags, void* stream) {
  if (n < 0 || !gauss6 || !props || !surf) return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: bad arguments");
  if (n == 0) return EB_OK;
  if (!d_in || !d_out || !d_flags) return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: null device buffer");
  cudaStream_t st = (cudaStream_t)stream;
  Gauss3 g;
  for (int i = 0; i < 3; ++i) { g.w[i] = gauss6[i]; g.z[i] = gauss6[3 + i]; }
  ContactProps cp{props[0], props[1], props[2], props[3]};
  // surface kind (0 sphere, 1 SDF, 2 plane) and the plane's axis are whole numbers in range
  // before they are converted
  if (!(surf[0] == 0 || surf[0] == 1 || surf[0] == 2) ||
      (surf[0] == 2 && !(surf[1] == 0 || surf[1] == 1 || surf[1] == 2)))
    return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: bad surface kind or plane axis");
  SurfaceDev s;
  std::memset(&s, 0, sizeof(s));
  s.kind = (int)surf[0];
  s.cx = surf[1]; s.cy = surf[2]; s.cz = surf[3]; s.R = surf[4];
  if (s.kind == 2) {
    s.axis = (int)surf[1];
    s.pos = surf[2];
  }
  if (s.kind == 1) {
    if (!d_sdf_values) return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: SDF values missing");
    // every grid dimension is checked on its own (finite, at least 1, within the array) before
    // the padded product is formed, so the product cannot overflow
    const double lim = (double)EB_NOALLOC_SDF_MAX_COEFS;
    for (int a = 5; a < 8; ++a)
      if (!std::isfinite(surf[a]) || !(surf[a] >= 1) || !(surf[a] <= lim) || surf[a] != std::floor(surf[a]))
        return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: bad SDF grid dimension (surf[5..7] must be "
                                            "integers in [1, EB_NOALLOC_SDF_MAX_COEFS])");
    for (int a = 8; a < 14; ++a)
      if (!std::isfinite(surf[a]) || (a >= 11 && !(surf[a] > 0)))
        return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: bad SDF origin or spacing (surf[8..13])");
    const int64_t nx = (int64_t)surf[5], ny = (int64_t)surf[6], nz = (int64_t)surf[7];
    if ((nx + 2) > (int64_t)EB_NOALLOC_SDF_MAX_COEFS / ((ny + 2) * (nz + 2)) ||
        (nx + 2) * (ny + 2) * (nz + 2) > (int64_t)EB_NOALLOC_SDF_MAX_COEFS)
      return eb_internal_fail(EB_ERR_ARG,
                              "eb_contact_eval_noalloc: SDF grid too large for the fixed coefficient array "
                              "((nx+2)(ny+2)(nz+2) > EB_NOALLOC_SDF_MAX_COEFS = 287496)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return err("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return eb_internal_fail(EB_ERR_ARG, "eb_contact_eval_noalloc: device ordinal");
    double* coef = nullptr;
    {
      std::lock_guard<std::mutex> lk(g_noalloc_mu);
      void* ctx = current_context();
      if (!g_noalloc_ptr[dev] || !ctx || ctx != g_noalloc_ctx[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_coef);
        if (e != cudaSuccess) return err("cudaGetSymbolAddress", e);
        g_noalloc_ptr[dev] = (double*)p;
        g_noalloc_ctx[dev] = current_context();
      }
      coef = g_noalloc_ptr[dev];
    }
    const int NX = (int)nx, NY = (int)ny, NZ = (int)nz;
    const int64_t pts = nx * ny * nz;
    k_sdf_interior<<<(unsigned)((pts + 255) / 256), 256, 0, st>>>(d_sdf_values, NX, NY, NZ, coef);
    k_sdf_prefilter_axis<<<(unsigned)((ny * nz + 127) / 128), 128, 0, st>>>(coef, NX, NY, NZ, 0);
    k_sdf_prefilter_axis<<<(unsigned)(((nx + 2) * nz + 127) / 128), 128, 0, st>>>(coef, NX, NY, NZ, 1);
    k_sdf_prefilter_axis<<<(unsigned)(((nx + 2) * (ny + 2) + 127) / 128), 128, 0, st>>>(coef, NX, NY, NZ, 2);
    s.coef = coef;
    s.nx = NX; s.ny = NY; s.nz = NZ;
    s.x0 = surf[8]; s.y0 = surf[9]; s.z0 = surf[10];
    s.ihx = 1.0 / surf[11]; s.ihy = 1.0 / surf[12]; s.ihz = 1.0 / surf[13];
    s.xl = (NX - 1) * surf[11]; s.yl = (NY - 1) * surf[12]; s.zl = (NZ - 1) * surf[13];
  }
  // untouched elements leave zero records, as in eb_contact_eval
  cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(double) * 301 * n, st);
  if (e != cudaSuccess) return err("cudaMemsetAsync", e);
  k_contact_eval<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, d_in, g, cp, s, d_out, d_flags);
  e = cudaGetLastError();
  if (e != cudaSuccess) return err("k_contact_eval (no-alloc) launch", e);
  return EB_OK;
}

// ---------------------------------------------------------------- FP64 throughput probe
namespace {
__global__ void k_fp64_fma(double* out, int iters, double b, double c) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}
}  // namespace

extern "C" int eb_fp64_peak(double* tflops) {
  if (!tflops) return EB_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8, iters = 4096;
  DBuf out;
  cudaError_t e;
  if ((e = cudaMalloc(&out.p, sizeof(double) * threads * blocks)) != cudaSuccess) return err("cudaMalloc", e);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fp64_fma<<<blocks, threads>>>((double*)out.p, iters, 0.999999, 1e-7);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(a);
    k_fp64_fma<<<blocks, threads>>>((double*)out.p, iters, 0.999999, 1e-7);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if ((e = cudaGetLastError()) != cudaSuccess) return err("k_fp64_fma", e);
  const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return EB_OK;
}
