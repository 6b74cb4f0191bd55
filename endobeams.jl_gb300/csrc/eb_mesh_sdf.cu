// Signed distance field of a closed triangle mesh on a regular grid.
//
// No counterpart in the reference: its DiscreteSignedDistanceField reads a
// precomputed grid (read_vtk_sdf, src/IO/read_input_files.jl:154-195), while
// its vessel geometries exist as triangle meshes (read_vtk_triangle_mesh,
// :81-152).  This turns such a mesh into the grid the contact kernels use.
//
// One thread per grid point; triangles stream through shared memory in tiles
// that every thread of the CTA shares.  Per (point, triangle):
//   * squared distance to the closest point of the triangle, by the Voronoi-
//     region tests of Ericson, "Real-Time Collision Detection" (2005), §5.1.5;
//   * the triangle's signed solid angle seen from the point, by the formula of
//     Van Oosterom & Strackee, IEEE Trans. Biomed. Eng. 30 (1983) 125-126:
//     tan(Ω/2) = a·(b×c) / (|a||b||c| + (a·b)|c| + (a·c)|b| + (b·c)|a|).
// The solid angles sum to 4π times the generalized winding number; the point is
// inside when |Σ Ω| > 2π (either orientation of the mesh).  The value is the
// distance, positive inside and negative outside — the sign convention of the
// reference's SDF files for bodies inside the surface (DiscreteSignedDistanceField
// with inside = true, def_interactions.jl:67-71).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/endobeams_gb300.h"

int eb_internal_fail(int code, const char* msg);  // sets eb_last_error (eb_abi.cu)

namespace {

constexpr int kSdfThreads = 128;
constexpr int kTile = 128;  // triangles per shared-memory tile (9 doubles each: 9 KB)

struct P3 {
  double x, y, z;
};
__device__ __forceinline__ P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ P3 cross(P3 a, P3 b) {
  return P3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ P3 axpy(double s, P3 a, P3 b) { return P3{b.x + s * a.x, b.y + s * a.y, b.z + s * a.z}; }

// Squared distance from p to triangle abc (closest-point region tests).
__device__ double dist2_point_triangle(P3 p, P3 a, P3 b, P3 c) {
  const P3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
  const double d1 = dot(ab, ap), d2 = dot(ac, ap);
  P3 q;
  if (d1 <= 0.0 && d2 <= 0.0) {
    q = a;  // vertex region a
  } else {
    const P3 bp = sub(p, b);
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) {
      q = b;  // vertex region b
    } else {
      const double vc = d1 * d4 - d3 * d2;
      if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        q = axpy(d1 / (d1 - d3), ab, a);  // edge ab
      } else {
        const P3 cp = sub(p, c);
        const double d5 = dot(ab, cp), d6 = dot(ac, cp);
        if (d6 >= 0.0 && d5 <= d6) {
          q = c;  // vertex region c
        } else {
          const double vb = d5 * d2 - d1 * d6;
          if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
            q = axpy(d2 / (d2 - d6), ac, a);  // edge ac
          } else {
            const double va = d3 * d6 - d5 * d4;
            if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
              q = axpy((d4 - d3) / ((d4 - d3) + (d5 - d6)), sub(c, b), b);  // edge bc
            } else {
              const double den = 1.0 / (va + vb + vc);  // face region
              const double v = vb * den, w = vc * den;
              q = axpy(w, ac, axpy(v, ab, a));
            }
          }
        }
      }
    }
  }
  const P3 d = sub(p, q);
  return dot(d, d);
}

// Signed solid angle of triangle abc seen from p.
__device__ double solid_angle(P3 p, P3 A, P3 B, P3 C) {
  const P3 a = sub(A, p), b = sub(B, p), c = sub(C, p);
  const double la = sqrt(dot(a, a)), lb = sqrt(dot(b, b)), lc = sqrt(dot(c, c));
  const double num = dot(a, cross(b, c));
  const double den = la * lb * lc + dot(a, b) * lc + dot(a, c) * lb + dot(b, c) * la;
  return 2.0 * atan2(num, den);
}

__global__ void __launch_bounds__(kSdfThreads) k_mesh_sdf(const double* __restrict__ tri, int64_t nt, int64_t nx,
                                                          int64_t ny, int64_t nz, double ox, double oy, double oz,
                                                          double hx, double hy, double hz, double* __restrict__ out) {
  __shared__ double st[kTile * 9];
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = nx * ny * nz;
  const bool valid = idx < N;
  P3 p{0.0, 0.0, 0.0};
  if (valid) {
    const int64_t i = idx % nx, j = (idx / nx) % ny, k = idx / (nx * ny);
    p = P3{ox + (double)i * hx, oy + (double)j * hy, oz + (double)k * hz};
  }
  double d2 = INFINITY, omega = 0.0;
  for (int64_t t0 = 0; t0 < nt; t0 += kTile) {
    const int cnt = (int)(nt - t0 < kTile ? nt - t0 : kTile);
    for (int q = threadIdx.x; q < cnt * 9; q += blockDim.x) st[q] = tri[t0 * 9 + q];
    __syncthreads();
    if (valid) {
      for (int t = 0; t < cnt; ++t) {
        const double* v = st + 9 * t;
        const P3 a{v[0], v[1], v[2]}, b{v[3], v[4], v[5]}, c{v[6], v[7], v[8]};
        d2 = fmin(d2, dist2_point_triangle(p, a, b, c));
        omega += solid_angle(p, a, b, c);
      }
    }
    __syncthreads();
  }
  if (valid) {
    const double d = sqrt(d2);
    out[idx] = fabs(omega) > 6.283185307179586 ? d : -d;  // |winding number| > 1/2: inside
  }
}

struct Buf {
  void* p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" int eb_sdf_from_mesh(int64_t n_vert, const double* verts, int64_t n_tri, const int64_t* tris,
                                const int64_t* dims, const double* origin, const double* spacing, double* out) {
  if (n_vert < 3 || n_tri < 1 || !verts || !tris || !dims || !origin || !spacing || !out)
    return eb_internal_fail(EB_ERR_ARG, "eb_sdf_from_mesh: bad arguments");
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || !(spacing[0] > 0) || !(spacing[1] > 0) || !(spacing[2] > 0))
    return eb_internal_fail(EB_ERR_ARG, "eb_sdf_from_mesh: bad grid");
  std::vector<double> tv(9 * (size_t)n_tri);
  for (int64_t t = 0; t < n_tri; ++t)
    for (int k = 0; k < 3; ++k) {
      const int64_t v = tris[3 * t + k];
      if (v < 0 || v >= n_vert) return eb_internal_fail(EB_ERR_ARG, "eb_sdf_from_mesh: triangle vertex out of range");
      std::memcpy(&tv[9 * t + 3 * k], verts + 3 * v, 3 * sizeof(double));
    }
  const int64_t N = dims[0] * dims[1] * dims[2];
  Buf dt, dout;
  if (cudaMalloc(&dt.p, sizeof(double) * tv.size()) != cudaSuccess ||
      cudaMalloc(&dout.p, sizeof(double) * (size_t)N) != cudaSuccess ||
      cudaMemcpy(dt.p, tv.data(), sizeof(double) * tv.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return eb_internal_fail(EB_ERR_CUDA, "eb_sdf_from_mesh: device allocation or copy failed");
  const unsigned blocks = (unsigned)((N + kSdfThreads - 1) / kSdfThreads);
  k_mesh_sdf<<<blocks, kSdfThreads>>>((const double*)dt.p, n_tri, dims[0], dims[1], dims[2], origin[0], origin[1],
                                      origin[2], spacing[0], spacing[1], spacing[2], (double*)dout.p);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpy(out, dout.p, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost) != cudaSuccess)
    return eb_internal_fail(EB_ERR_CUDA, "eb_sdf_from_mesh: kernel or copy failed");
  return EB_OK;
}
