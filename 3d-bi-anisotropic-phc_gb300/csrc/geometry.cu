// Vertex rasterisation of the inclusions on the device: which grid vertices
// lie inside the woodpile rods, a sphere or a regular tetrahedron (with their
// periodic images).  Replaces the host-side point location of
// subroutines/Material_Locate_Isofunction.m:1-28 with the isofunctions of
// Public/woodpile_isofun.m:1-13, the sphere isofunction of
// InputData/BS_Gyroid/Physical_settings_sphere.m:18 and the same-side-of-
// plane test of subroutines/Material_Locate_Isofunction.m:135-148.
//
// Every floating-point step is an explicitly rounded intrinsic in the order
// the reference's expressions give (no contraction into FMA), so the ids are
// the ones a host evaluation of the same expressions in IEEE double gives.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>

#include "fame_internal.h"

namespace fame {
namespace {

constexpr int kImages = 27;  // periodic images i, j, k in {-1, 0, 1}

struct GeomArgs {
  int n;
  int shape;
  int id;
  int paint;
  double A[9];   // primitive vectors as columns, row-major
  double p[4];   // shape parameters
};

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// Cartesian position of vertex (i1, i2, i3): lattice coefficients (i-1)/n
// (Public/Grid_Generate_Mult_Point.m:7-17) times A', summed left to right.
__device__ __forceinline__ void vertex_pos(const GeomArgs& g, int i1, int i2, int i3, double P[3]) {
  const double c1 = ddiv((double)i1, (double)g.n);
  const double c2 = ddiv((double)i2, (double)g.n);
  const double c3 = ddiv((double)i3, (double)g.n);
#pragma unroll
  for (int r = 0; r < 3; ++r)
    P[r] = dadd(dadd(dmul(c1, g.A[r * 3 + 0]), dmul(c2, g.A[r * 3 + 1])), dmul(c3, g.A[r * 3 + 2]));
}

// Public/woodpile_isofun.m:7-11 with w -> sqrt(2)/2*w.
__device__ __forceinline__ bool woodpile_inside(const double P[3], double width, double a) {
  const double x = P[0], y = P[1], z = P[2];
  const double t1 = dsub(y, x), t2 = dadd(y, x);
  const double w = dmul(ddiv(__dsqrt_rn(2.0), 2.0), width);
  const double a4 = ddiv(a, 4.0), a2 = ddiv(a, 2.0), a34 = ddiv(dmul(3.0, a), 4.0);
  const double a32 = ddiv(dmul(3.0, a), 2.0), a2x = dmul(2.0, a);
  const bool l0 = (z >= 0.0 && z < a4) &&
                  (t1 >= dsub(a, w) || t1 <= -dsub(a, w) || (t1 >= -w && t1 <= w));
  const bool l1 = (z >= a4 && z < a2) &&
                  ((t2 >= dsub(a32, w) && t2 <= dadd(a32, w)) || (t2 >= dsub(a2, w) && t2 <= dadd(a2, w)));
  const bool l2 = (z >= a2 && z < a34) &&
                  ((t1 >= dsub(-a2, w) && t1 <= dadd(-a2, w)) || (t1 >= dsub(a2, w) && t1 <= dadd(a2, w)));
  const bool l3 = (z >= a34 && z <= a) &&
                  (t2 >= dsub(a2x, w) || t2 <= w || (t2 >= dsub(a, w) && t2 <= dadd(a, w)));
  return l0 || l1 || l2 || l3;
}

// Image offset A [i j k]' of image m (i, j, k = m/9 - 1, (m/3)%3 - 1, m%3 - 1).
__device__ __forceinline__ void image_offset(const GeomArgs& g, int m, double o[3]) {
  const double i = (double)(m / 9 - 1), j = (double)((m / 3) % 3 - 1), k = (double)(m % 3 - 1);
#pragma unroll
  for (int r = 0; r < 3; ++r)
    o[r] = dadd(dadd(dmul(g.A[r * 3 + 0], i), dmul(g.A[r * 3 + 1], j)), dmul(g.A[r * 3 + 2], k));
}

// Regular tetrahedron: vertices s*(1,1,1), s*(1,-1,-1), s*(-1,1,-1),
// s*(-1,-1,1) about the centre, s = edge/(2 sqrt 2).
__device__ __forceinline__ void tetra_vertex(const GeomArgs& g, int t, const double off[3], double v[3]) {
  const double s = ddiv(g.p[0], dmul(2.0, __dsqrt_rn(2.0)));
  const double sg[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
#pragma unroll
  for (int r = 0; r < 3; ++r) v[r] = dadd(dadd(dmul(s, sg[t][r]), g.p[1 + r]), off[r]);
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return dadd(dadd(dmul(a[0], b[0]), dmul(a[1], b[1])), dmul(a[2], b[2]));
}

// Per image and face of the tetrahedron: a point a of the face, the face
// normal cross(b - a, c - a) and the sign side of the opposite vertex q.
struct Face {
  double a[3], nrm[3], dq;
};

__global__ void k_rasterize(GeomArgs g, uint8_t* __restrict__ phase) {
  __shared__ double centre[kImages][3];
  __shared__ Face face[kImages * 4];
  const int tid = threadIdx.x;
  if (g.shape == FAME_SHAPE_SPHERE && tid < kImages) {
    double off[3];
    image_offset(g, tid, off);
#pragma unroll
    for (int r = 0; r < 3; ++r) centre[tid][r] = dadd(g.p[1 + r], off[r]);
  }
  if (g.shape == FAME_SHAPE_TETRA && tid < kImages * 4) {
    const int m = tid / 4, f = tid % 4;
    double off[3], v[4][3];
    image_offset(g, m, off);
#pragma unroll
    for (int t = 0; t < 4; ++t) tetra_vertex(g, t, off, v[t]);
    const int ia = f == 0 ? 1 : 0, ib = f <= 1 ? 2 : 1, ic = f <= 2 ? 3 : 2;  // the three t != f
    double ba[3], ca[3], qa[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      ba[r] = dsub(v[ib][r], v[ia][r]);
      ca[r] = dsub(v[ic][r], v[ia][r]);
      qa[r] = dsub(v[ia][r], v[f][r]);
    }
    Face& F = face[tid];
    F.nrm[0] = dsub(dmul(ba[1], ca[2]), dmul(ba[2], ca[1]));
    F.nrm[1] = dsub(dmul(ba[2], ca[0]), dmul(ba[0], ca[2]));
    F.nrm[2] = dsub(dmul(ba[0], ca[1]), dmul(ba[1], ca[0]));
#pragma unroll
    for (int r = 0; r < 3; ++r) F.a[r] = v[ia][r];
    F.dq = dot3(qa, F.nrm);
  }
  __syncthreads();
  const long long Nq = (long long)g.n * g.n * g.n;
  for (long long v = (long long)blockIdx.x * blockDim.x + tid; v < Nq; v += (long long)gridDim.x * blockDim.x) {
    const int i1 = (int)(v % g.n), i2 = (int)((v / g.n) % g.n), i3 = (int)(v / ((long long)g.n * g.n));
    double P[3];
    vertex_pos(g, i1, i2, i3, P);
    bool in = false;
    if (g.shape == FAME_SHAPE_WOODPILE) {
      in = woodpile_inside(P, g.p[0], g.p[1]);
    } else if (g.shape == FAME_SHAPE_SPHERE) {
      // -min_c |r - c| > -radius  (Physical_settings_sphere.m:18 with isoval -radius)
      double best = INFINITY;
      for (int m = 0; m < kImages; ++m) {
        const double dx = dsub(P[0], centre[m][0]), dy = dsub(P[1], centre[m][1]), dz = dsub(P[2], centre[m][2]);
        const double d = __dsqrt_rn(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)));
        best = fmin(best, d);
      }
      in = -best > -g.p[0];
    } else {
      // pointSideOfPlane for the four faces (Material_Locate_Isofunction.m:135-148)
      const double tol = 1e-8;
      for (int m = 0; m < kImages && !in; ++m) {
        bool ok = true;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          const Face& F = face[m * 4 + f];
          const double pa[3] = {dsub(F.a[0], P[0]), dsub(F.a[1], P[1]), dsub(F.a[2], P[2])};
          const double dp = dot3(pa, F.nrm);
          ok = ok && (fabs(dp) < tol || fabs(F.dq) < tol || dmul(dp, F.dq) > 0.0);
        }
        in = ok;
      }
    }
    if (in)
      phase[v] = (uint8_t)g.id;
    else if (!g.paint)
      phase[v] = 0;
  }
}

}  // namespace
}  // namespace fame

extern "C" {

int fame_rasterize(int n, const double* lattice, int shape, const double* params, int id, uint8_t* phase,
                   int flags) {
  using namespace fame;
  if (n < 1 || n > 2048 || !lattice || !params || !phase || id < 0 || id > 255)
    return fail(nullptr, FAME_ERR_BAD_ARG, "fame_rasterize: bad argument");
  GeomArgs g{};
  g.n = n;
  g.shape = shape;
  g.id = id;
  g.paint = (flags & FAME_RASTER_PAINT) ? 1 : 0;
  for (int i = 0; i < 9; ++i) g.A[i] = lattice[i];
  int np = 0;
  switch (shape) {
    case FAME_SHAPE_WOODPILE: np = 2; break;
    case FAME_SHAPE_SPHERE:
    case FAME_SHAPE_TETRA: np = 4; break;
    default: return fail(nullptr, FAME_ERR_BAD_ARG, "fame_rasterize: unknown shape " + std::to_string(shape));
  }
  for (int i = 0; i < np; ++i) {
    g.p[i] = params[i];
    if (!std::isfinite(g.p[i])) return fail(nullptr, FAME_ERR_BAD_ARG, "fame_rasterize: non-finite parameter");
  }
  if (!(g.p[0] > 0.0) || (shape == FAME_SHAPE_WOODPILE && !(g.p[1] > 0.0)))
    return fail(nullptr, FAME_ERR_BAD_ARG, "fame_rasterize: size parameters must be positive");
  for (int i = 0; i < 9; ++i)
    if (!std::isfinite(g.A[i])) return fail(nullptr, FAME_ERR_BAD_ARG, "fame_rasterize: non-finite lattice");

  const size_t Nq = (size_t)n * n * n;
  const bool host = (flags & FAME_HOST_PTR) != 0;
  uint8_t* dbuf = nullptr;  // device staging of a host array
  cudaError_t e = cudaSuccess;
  if (host) {
    void* tmp = nullptr;
    e = cudaMalloc(&tmp, Nq);
    if (e == cudaSuccess) dbuf = (uint8_t*)tmp;
    if (e == cudaSuccess && g.paint) e = cudaMemcpy(dbuf, phase, Nq, cudaMemcpyHostToDevice);
  }
  uint8_t* d = host ? dbuf : phase;
  if (e == cudaSuccess) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tpb = 256;
    long long blocks = ((long long)Nq + tpb - 1) / tpb;
    const long long cap = 8LL * (sms > 0 ? sms : 1);
    if (blocks > cap) blocks = cap;
    FAME_LAUNCHED(1);
    k_rasterize<<<(unsigned)blocks, tpb>>>(g, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = host ? cudaMemcpy(phase, d, Nq, cudaMemcpyDeviceToHost) : cudaDeviceSynchronize();
  if (dbuf) cudaFree(dbuf);
  if (e != cudaSuccess) return fail(nullptr, FAME_ERR_CUDA, std::string("fame_rasterize: ") + cudaGetErrorString(e));
  return FAME_OK;
}

}  // extern "C"
