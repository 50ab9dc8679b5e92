// Material stencil of fncB on the six spatial fields (periodic frame):
//   stage 1 (k_vertex)  : U_j, V_j gathered to every vertex, Hu, Hv = vertex
//                         tensor products  -> scratch h
//   stage 2 (k_faceedge): u'_i = m_i u_i + 1/4 (I+T_a)(I+T_b) Hu_i,
//                         v'_i = n_i v_i + 1/2 (I+T_i) Hv_i   (in place)
// One thread per vertex / voxel.  Size templated (instantiated per grid size
// with the transforms in fncb_inst_*.cu) so that the index arithmetic is
// 32-bit with compile-time divisors.
//
// A fused single-kernel form (tiles with a one-voxel halo in shared memory)
// reads and writes each field once instead of three / two times, but it
// recomputes stage 1 on the halo; at n = 60 that cost more issue slots than
// the DRAM traffic it saved, so the two-kernel form is kept.
#pragma once

#include "fame_internal.h"

namespace fame {
namespace detail {

template <class R> inline const PlanData<R>& pdata(const Plan& P);
template <> inline const PlanData<double>& pdata<double>(const Plan& P) { return P.d64; }
template <> inline const PlanData<float>& pdata<float>(const Plan& P) { return P.d32; }
template <> inline const PlanData<ff>& pdata<ff>(const Plan& P) { return P.dds; }

template <class R, int N>
__global__ void __launch_bounds__(512)
k_vertex(const cx<R>* __restrict__ uv, cx<R>* __restrict__ h, PlanData<R> d,
         const uint8_t* __restrict__ phase, int nphase, VecCtx ctx, long long stride) {
  constexpr int NN = N * N, Nq = NN * N;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = idx % N, i2 = (idx / N) % N, i3 = idx / NN;
  const int dxm = i1 == 0 ? N - 1 : -1;
  const int dym = i2 == 0 ? (N - 1) * N : -N;
  const int dzm = i3 == 0 ? (N - 1) * NN : -NN;
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> tx = cconj(tau[0]), ty = cconj(tau[1]), tz = cconj(tau[2]);
  const cx<R>* f = uv + vec * stride + idx;
  // U_j = 1/4 (I + T_a^H)(I + T_b^H) u_j ; (T^H g)(r) = conj(tau) g(r - e)
  auto face2vtx = [&](const cx<R>* g, int da, int db, cx<R> ta, cx<R> tb) {
    cx<R> s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    return cscale(s, R(0.25));
  };
  cx<R> U[3], V[3];
  U[0] = face2vtx(f, dym, dzm, ty, tz);
  U[1] = face2vtx(f + Nq, dxm, dzm, tx, tz);
  U[2] = face2vtx(f + 2 * Nq, dxm, dym, tx, ty);
  V[0] = cscale(cfma(tx, f[3 * Nq + dxm], f[3 * Nq]), R(0.5));
  V[1] = cscale(cfma(ty, f[4 * Nq + dym], f[4 * Nq]), R(0.5));
  V[2] = cscale(cfma(tz, f[5 * Nq + dzm], f[5 * Nq]), R(0.5));
  cx<R>* o = h + vec * stride + idx;
  if (d.fld) {  // field mode: Mh = b G, Nh = a G, J = -i g G
    const R a = d.fld[idx], b = d.fld[Nq + idx], g = d.fld[2 * Nq + idx];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      cx<R> su = zero<R>(), sv = zero<R>();
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if (j != i) {
          su = cadd(su, cscale(U[j], d.gram[i * 3 + j]));
          sv = cadd(sv, cscale(V[j], d.gram[i * 3 + j]));
        }
      const cx<R> tu = cadd(su, cscale(U[i], d.gram[i * 4])), tv = cadd(sv, cscale(V[i], d.gram[i * 4]));
      // Hu_i = b sum_{j!=i} G_ij U_j + i g sum_j G_ij V_j ; Hv_i = a sum_{j!=i} G_ij V_j - i g sum_j G_ij U_j
      o[i * Nq] = cadd(cscale(su, b), cscale(cmul_i<+1>(tv), g));
      o[(3 + i) * Nq] = cadd(cscale(sv, a), cscale(cmul_i<-1>(tu), g));
    }
    return;
  }
  const cx<R>* T = d.mat + (inst * nphase + __ldg(phase + idx)) * 27;
  const cx<R>* Nh = T;
  const cx<R>* Mh = T + 9;
  const cx<R>* J = T + 18;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    cx<R> hu = zero<R>(), hv = zero<R>();
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j != i) {
        hu = cfma(Mh[i * 3 + j], U[j], hu);
        hv = cfma(Nh[i * 3 + j], V[j], hv);
      }
      hu = cfmac(J[j * 3 + i], V[j], hu);
      hv = cfma(J[i * 3 + j], U[j], hv);
    }
    o[i * Nq] = hu;
    o[(3 + i) * Nq] = hv;
  }
}

template <class R, int N>
__global__ void __launch_bounds__(512)
k_faceedge(cx<R>* __restrict__ uv, const cx<R>* __restrict__ h, PlanData<R> d,
           const uint8_t* __restrict__ phase, int nphase, VecCtx ctx, long long stride) {
  constexpr int NN = N * N, Nq = NN * N;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = idx % N, i2 = (idx / N) % N, i3 = idx / NN;
  const int dxp = i1 == N - 1 ? -(N - 1) : 1;
  const int dyp = i2 == N - 1 ? -(N - 1) * N : N;
  const int dzp = i3 == N - 1 ? -(N - 1) * NN : NN;
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> tx = tau[0], ty = tau[1], tz = tau[2];
  // material diagonals at the corners r + {0,1}^3
  R m0, m1, m2, n0, n1, n2;
  if (d.fld) {  // field mode: Re Mh_ii = b G_ii, Re Nh_ii = a G_ii
    const R* fa = d.fld + idx;
    const R* fb = d.fld + Nq + idx;
    m0 = R(0.25) * d.gram[0] * (fb[0] + fb[dyp] + fb[dzp] + fb[dyp + dzp]);
    m1 = R(0.25) * d.gram[4] * (fb[0] + fb[dxp] + fb[dzp] + fb[dxp + dzp]);
    m2 = R(0.25) * d.gram[8] * (fb[0] + fb[dxp] + fb[dyp] + fb[dxp + dyp]);
    n0 = R(0.5) * d.gram[0] * (fa[0] + fa[dxp]);
    n1 = R(0.5) * d.gram[4] * (fa[0] + fa[dyp]);
    n2 = R(0.5) * d.gram[8] * (fa[0] + fa[dzp]);
  } else {
    const cx<R>* tab = d.mat + inst * nphase * 27;
    const uint8_t* ph = phase + idx;
    const int p000 = __ldg(ph), p100 = __ldg(ph + dxp), p010 = __ldg(ph + dyp), p001 = __ldg(ph + dzp);
    const int p110 = __ldg(ph + dxp + dyp), p101 = __ldg(ph + dxp + dzp), p011 = __ldg(ph + dyp + dzp);
    auto reM = [&](int p, int i) { return tab[p * 27 + 9 + i * 4].x; };
    auto reN = [&](int p, int i) { return tab[p * 27 + i * 4].x; };
    m0 = R(0.25) * (reM(p000, 0) + reM(p010, 0) + reM(p001, 0) + reM(p011, 0));
    m1 = R(0.25) * (reM(p000, 1) + reM(p100, 1) + reM(p001, 1) + reM(p101, 1));
    m2 = R(0.25) * (reM(p000, 2) + reM(p100, 2) + reM(p010, 2) + reM(p110, 2));
    n0 = R(0.5) * (reN(p000, 0) + reN(p100, 0));
    n1 = R(0.5) * (reN(p000, 1) + reN(p010, 1));
    n2 = R(0.5) * (reN(p000, 2) + reN(p001, 2));
  }
  const cx<R>* hh = h + vec * stride + idx;
  cx<R>* f = uv + vec * stride + idx;
  // u'_i = m_i u_i + 1/4 (I+T_a)(I+T_b) Hu_i ; (T g)(r) = tau g(r + e)
  auto vtx2face = [&](const cx<R>* g, int da, int db, cx<R> ta, cx<R> tb) {
    cx<R> s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    return cscale(s, R(0.25));
  };
  cx<R> r[6];
  r[0] = cadd(cscale(f[0], m0), vtx2face(hh, dyp, dzp, ty, tz));
  r[1] = cadd(cscale(f[Nq], m1), vtx2face(hh + Nq, dxp, dzp, tx, tz));
  r[2] = cadd(cscale(f[2 * Nq], m2), vtx2face(hh + 2 * Nq, dxp, dyp, tx, ty));
  const cx<R>* hv = hh + 3 * Nq;
  r[3] = cadd(cscale(f[3 * Nq], n0), cscale(cfma(tx, hv[dxp], hv[0]), R(0.5)));
  r[4] = cadd(cscale(f[4 * Nq], n1), cscale(cfma(ty, hv[Nq + dyp], hv[Nq]), R(0.5)));
  r[5] = cadd(cscale(f[5 * Nq], n2), cscale(cfma(tz, hv[2 * Nq + dzp], hv[2 * Nq]), R(0.5)));
#pragma unroll
  for (int c = 0; c < 6; ++c) f[c * Nq] = r[c];
}

// ---------------------------------------------------------------------------
// Single-pass form of the same stencil: k_sweep reads the six spatial fields
// once and writes u', v' to a separate buffer, with no vertex scratch in
// global memory.  One CTA owns TY rows (all x) of a chunk of TZ consecutive
// z-planes of one vector and sweeps through the chunk plane by plane:
//   * the fields of plane z (rows y0-1 .. y0+TY, all six) are staged in
//     shared memory by cp.async, one plane ahead of the plane being computed
//     (three plane buffers);
//   * stage 1 evaluates U, V and the vertex products Hu, Hv of plane z on
//     rows y0 .. y0+TY (the one extra row is the +y neighbour the scatter
//     needs) from planes z and z-1, together with the real diagonals
//     D = (Re Mh_00, Re Mh_11, Re Mh_22, Re Nh_00, Re Nh_11, Re Nh_22) of
//     each vertex (the lumped m_i, n_i are face / edge averages of D);
//   * stage 2 then completes plane z-1 from the vertex values of planes z-1
//     and z.
// The chunk reads TZ+2 planes and evaluates stage 1 on TZ+1 planes for TZ
// output planes; in y, TY+2 rows are read and TY+1 evaluated for TY written.
// ---------------------------------------------------------------------------
template <class R, int N> struct SweepShape {
  static constexpr int ty_pick() {
    if constexpr (sizeof(R) == 8) return N % 2 == 0 ? 2 : 1;
    else return N % 4 == 0 ? 4 : N % 3 == 0 ? 3 : N % 2 == 0 ? 2 : 1;
  }
  static constexpr int tz_pick() {
    for (int t = 15; t >= 1; --t)
      if (N % t == 0) return t;
    return 1;
  }
  static constexpr int TY = ty_pick();
  static constexpr int TZ = tz_pick();
  static constexpr int FR = TY + 2;                       // staged field rows
  static constexpr int HR = TY + 1;                       // vertex rows
  static constexpr int TPB = (((HR * N + 31) / 32) * 32) > 512 ? 512 : (((HR * N + 31) / 32) * 32);
  static constexpr size_t F_ELEMS = 6 * FR * N;           // one staged plane (complex)
  static constexpr size_t H_ELEMS = 6 * HR * N;           // vertex values of one plane (complex)
  static constexpr int TAB_MAX = 8;                      // phases whose tensors are staged in shared memory
  static constexpr size_t SMEM = sizeof(cx<R>) * (3 * F_ELEMS + 2 * H_ELEMS + TAB_MAX * 27) + sizeof(R) * 2 * H_ELEMS;
  static constexpr int CPR = int(N * sizeof(cx<R>) / 16);  // 16-byte chunks per row
  static constexpr int CH = 6 * FR * CPR;                   // 16-byte chunks per staged plane
  static constexpr int NCH = (CH + TPB - 1) / TPB;          // chunks per thread
  static_assert((N * sizeof(cx<R>)) % 16 == 0, "rows must be whole 16-byte chunks");
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}

template <class R, int N>
__global__ void __launch_bounds__(SweepShape<R, N>::TPB)
k_sweep(const cx<R>* __restrict__ uv, cx<R>* __restrict__ out, PlanData<R> d, const uint8_t* __restrict__ phase,
        int nphase, VecCtx ctx, long long stride, double2* __restrict__ wdot) {
  using SH = SweepShape<R, N>;
  constexpr int TY = SH::TY, TZ = SH::TZ, FR = SH::FR, HR = SH::HR, TPB = SH::TPB, CPR = SH::CPR;
  constexpr int NN = N * N, Nq = NN * N;
  constexpr int EPC = 16 / int(sizeof(cx<R>));             // complex per 16-byte chunk
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<R>* Fb = reinterpret_cast<cx<R>*>(smem_raw);            // [3][6][FR][N]
  cx<R>* Hb = Fb + 3 * SH::F_ELEMS;                          // [2][6][HR][N]
  cx<R>* Tb = Hb + 2 * SH::H_ELEMS;                          // [TAB_MAX][27] material tensors
  R* Db = reinterpret_cast<R*>(Tb + SH::TAB_MAX * 27);       // [2][6][HR][N]
  const int y0 = blockIdx.x * TY;
  const int z0 = blockIdx.y * TZ;
  const int vec = blockIdx.z;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int tid = threadIdx.x;
  const cx<R>* src = uv + vec * stride;
  cx<R>* dst = out + vec * stride;
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> Tx = tau[0], Ty = tau[1], Tz = tau[2];
  const cx<R> tx = cconj(Tx), ty = cconj(Ty), tz = cconj(Tz);
  // products of two shifts' phases (diagonal neighbours), once per CTA
  const cx<R> txty = cmul(tx, ty), txtz = cmul(tx, tz), tytz = cmul(ty, tz);
  const cx<R> TxTy = cmul(Tx, Ty), TxTz = cmul(Tx, Tz), TyTz = cmul(Ty, Tz);
  const cx<R>* tab = d.fld ? nullptr : d.mat + inst * nphase * 27;
  const bool tab_sm = !d.fld && nphase <= SH::TAB_MAX;
  if (tab_sm)
    for (int i = tid; i < nphase * 27; i += TPB) Tb[i] = tab[i];
  if (tab_sm) tab = Tb;

  // This thread's 16-byte chunks of a staged plane: shared-memory offset and
  // global offset within the plane, the same for every plane of the sweep.
  int soff[SH::NCH], goff[SH::NCH];
#pragma unroll
  for (int i = 0; i < SH::NCH; ++i) {
    const int c = tid + i * TPB;
    const int f = c / (FR * CPR);
    const int rem = c - f * (FR * CPR);
    const int r = rem / CPR;
    const int cc = rem - r * CPR;
    const int y = (y0 - 1 + r + N) % N;
    soff[i] = (f * FR + r) * N + cc * EPC;
    goff[i] = f * Nq + y * N + cc * EPC;
  }
  auto stage = [&](int s) {  // plane z0-1+s -> Fb[s % 3]
    const int z = (z0 - 1 + s + N) % N;
    cx<R>* F = Fb + (s % 3) * SH::F_ELEMS;
    const cx<R>* sp = src + z * NN;
#pragma unroll
    for (int i = 0; i < SH::NCH; ++i)
      if (i < SH::NCH - 1 || tid + i * TPB < SH::CH) cp_async16(F + soff[i], sp + goff[i]);
    cp_async_commit();
  };

  double acc = 0.0;  // sum of Re(conj(w) . out) over this CTA's outputs (wdot)
  // Each thread evaluates stage 1 at the same (row, x) of every plane, so its
  // vertex's phase id for the next plane is loaded one step ahead.
  const int h_hr = tid / N, h_x = tid - (tid / N) * N;
  const bool h_act = tid < HR * N;
  const int h_row = (y0 + h_hr) % N;
  int ph_next = 0;
  if (!d.fld && h_act) ph_next = __ldg(phase + ((z0 + N) % N) * NN + h_row * N + h_x);
  stage(0);
  for (int s = 0; s <= TZ + 1; ++s) {
    __syncthreads();  // readers of the buffers refilled below are done
    if (s + 1 <= TZ + 1) {
      stage(s + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // plane s is visible to every thread
    const int zc = (z0 - 1 + s + N) % N;
    if (s >= 1) {
      // stage 1 on plane zc, vertex rows y0 .. y0+TY
      const cx<R>* Fc = Fb + (s % 3) * SH::F_ELEMS;
      const cx<R>* Fp = Fb + ((s - 1) % 3) * SH::F_ELEMS;
      cx<R>* H = Hb + (s % 2) * SH::H_ELEMS;
      R* D = Db + (s % 2) * SH::H_ELEMS;
      if (h_act) {
        const int hr = h_hr;
        const int x = h_x;
        const int xm = x == 0 ? N - 1 : x - 1;
        const int rc = hr + 1, rm = hr;  // staged rows of y and y-1
        auto at = [&](const cx<R>* F, int f, int r, int xx) { return F[(f * FR + r) * N + xx]; };
        // U_j = 1/4 (I + T_a^H)(I + T_b^H) u_j ; (T^H g)(r) = conj(tau) g(r - e)
        auto g4 = [&](cx<R> g00, cx<R> ga, cx<R> gb, cx<R> gab, cx<R> ta, cx<R> tb, cx<R> tab2) {
          cx<R> s4 = g00;
          s4 = cfma(ta, ga, s4);
          s4 = cfma(tb, gb, s4);
          s4 = cfma(tab2, gab, s4);
          return cscale(s4, R(0.25));
        };
        cx<R> U[3], V[3];
        U[0] = g4(at(Fc, 0, rc, x), at(Fc, 0, rm, x), at(Fp, 0, rc, x), at(Fp, 0, rm, x), ty, tz, tytz);
        U[1] = g4(at(Fc, 1, rc, x), at(Fc, 1, rc, xm), at(Fp, 1, rc, x), at(Fp, 1, rc, xm), tx, tz, txtz);
        U[2] = g4(at(Fc, 2, rc, x), at(Fc, 2, rc, xm), at(Fc, 2, rm, x), at(Fc, 2, rm, xm), tx, ty, txty);
        V[0] = cscale(cfma(tx, at(Fc, 3, rc, xm), at(Fc, 3, rc, x)), R(0.5));
        V[1] = cscale(cfma(ty, at(Fc, 4, rm, x), at(Fc, 4, rc, x)), R(0.5));
        V[2] = cscale(cfma(tz, at(Fp, 5, rc, x), at(Fc, 5, rc, x)), R(0.5));
        const int vidx = zc * NN + h_row * N + x;
        cx<R> hu[3], hv[3];
        R dg[6];
        if (d.fld) {  // field mode: Mh = b G, Nh = a G, J = -i g G
          const R a = d.fld[vidx], b = d.fld[Nq + vidx], g = d.fld[2 * Nq + vidx];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            cx<R> su = zero<R>(), sv = zero<R>();
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (j != i) {
                su = cadd(su, cscale(U[j], d.gram[i * 3 + j]));
                sv = cadd(sv, cscale(V[j], d.gram[i * 3 + j]));
              }
            const cx<R> tu = cadd(su, cscale(U[i], d.gram[i * 4])), tv = cadd(sv, cscale(V[i], d.gram[i * 4]));
            hu[i] = cadd(cscale(su, b), cscale(cmul_i<+1>(tv), g));
            hv[i] = cadd(cscale(sv, a), cscale(cmul_i<-1>(tu), g));
            dg[i] = b * d.gram[i * 4];
            dg[3 + i] = a * d.gram[i * 4];
          }
        } else {
          const cx<R>* T = tab + ph_next * 27;
          ph_next = __ldg(phase + ((zc + 1) % N) * NN + h_row * N + x);  // the next plane's id, one step ahead
          const cx<R>* Nh = T;
          const cx<R>* Mh = T + 9;
          const cx<R>* J = T + 18;
          // Herm(N), Herm(M): the upper off-diagonal entries and their conjugates
          const cx<R> m01 = Mh[1], m02 = Mh[2], m12 = Mh[5];
          const cx<R> n01 = Nh[1], n02 = Nh[2], n12 = Nh[5];
          cx<R> Jr[9];
#pragma unroll
          for (int i = 0; i < 9; ++i) Jr[i] = J[i];
          // Hu_i = sum_{j!=i} Mh_ij U_j + sum_j conj(J_ji) V_j ; Hv_i = sum_{j!=i} Nh_ij V_j + sum_j J_ij U_j
          hu[0] = cfma(m01, U[1], cmul(m02, U[2]));
          hu[1] = cfmac(m01, U[0], cmul(m12, U[2]));
          hu[2] = cfmac(m02, U[0], cmulc(m12, U[1]));
          hv[0] = cfma(n01, V[1], cmul(n02, V[2]));
          hv[1] = cfmac(n01, V[0], cmul(n12, V[2]));
          hv[2] = cfmac(n02, V[0], cmulc(n12, V[1]));
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              hu[i] = cfmac(Jr[j * 3 + i], V[j], hu[i]);
              hv[i] = cfma(Jr[i * 3 + j], U[j], hv[i]);
            }
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            dg[i] = Mh[i * 4].x;
            dg[3 + i] = Nh[i * 4].x;
          }
        }
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          H[(f * HR + hr) * N + x] = hu[f];
          H[((3 + f) * HR + hr) * N + x] = hv[f];
        }
#pragma unroll
        for (int f = 0; f < 6; ++f) D[(f * HR + hr) * N + x] = dg[f];
      }
    }
    __syncthreads();
    if (s >= 2) {
      // stage 2 on plane zo = zc - 1 (vertex values of zo in slot s-1, of zc in slot s)
      const int zo = (zc - 1 + N) % N;
      const cx<R>* F = Fb + ((s - 1) % 3) * SH::F_ELEMS;
      const cx<R>* H0 = Hb + ((s - 1) % 2) * SH::H_ELEMS;
      const cx<R>* H1 = Hb + (s % 2) * SH::H_ELEMS;
      const R* D0 = Db + ((s - 1) % 2) * SH::H_ELEMS;
      const R* D1 = Db + (s % 2) * SH::H_ELEMS;
      for (int it = tid; it < TY * N; it += TPB) {
        const int r = it / N;
        const int x = it - r * N;
        const int xp = x == N - 1 ? 0 : x + 1;
        auto h = [&](const cx<R>* Hp, int f, int rr, int xx) { return Hp[(f * HR + rr) * N + xx]; };
        auto dd = [&](const R* Dp, int f, int rr, int xx) { return Dp[(f * HR + rr) * N + xx]; };
        // u'_i = m_i u_i + 1/4 (I+T_a)(I+T_b) Hu_i ; (T g)(r) = tau g(r + e)
        auto s4 = [&](cx<R> g00, cx<R> ga, cx<R> gb, cx<R> gab, cx<R> ta, cx<R> tb, cx<R> tab2) {
          cx<R> q = g00;
          q = cfma(ta, ga, q);
          q = cfma(tb, gb, q);
          q = cfma(tab2, gab, q);
          return cscale(q, R(0.25));
        };
        const R m0 = R(0.25) * (dd(D0, 0, r, x) + dd(D0, 0, r + 1, x) + dd(D1, 0, r, x) + dd(D1, 0, r + 1, x));
        const R m1 = R(0.25) * (dd(D0, 1, r, x) + dd(D0, 1, r, xp) + dd(D1, 1, r, x) + dd(D1, 1, r, xp));
        const R m2 = R(0.25) * (dd(D0, 2, r, x) + dd(D0, 2, r, xp) + dd(D0, 2, r + 1, x) + dd(D0, 2, r + 1, xp));
        const R n0 = R(0.5) * (dd(D0, 3, r, x) + dd(D0, 3, r, xp));
        const R n1 = R(0.5) * (dd(D0, 4, r, x) + dd(D0, 4, r + 1, x));
        const R n2 = R(0.5) * (dd(D0, 5, r, x) + dd(D1, 5, r, x));
        const int fr = r + 1;
        cx<R> o[6];
        o[0] = cadd(cscale(F[(0 * FR + fr) * N + x], m0),
                    s4(h(H0, 0, r, x), h(H0, 0, r + 1, x), h(H1, 0, r, x), h(H1, 0, r + 1, x), Ty, Tz, TyTz));
        o[1] = cadd(cscale(F[(1 * FR + fr) * N + x], m1),
                    s4(h(H0, 1, r, x), h(H0, 1, r, xp), h(H1, 1, r, x), h(H1, 1, r, xp), Tx, Tz, TxTz));
        o[2] = cadd(cscale(F[(2 * FR + fr) * N + x], m2),
                    s4(h(H0, 2, r, x), h(H0, 2, r, xp), h(H0, 2, r + 1, x), h(H0, 2, r + 1, xp), Tx, Ty, TxTy));
        o[3] = cadd(cscale(F[(3 * FR + fr) * N + x], n0), cscale(cfma(Tx, h(H0, 3, r, xp), h(H0, 3, r, x)), R(0.5)));
        o[4] = cadd(cscale(F[(4 * FR + fr) * N + x], n1), cscale(cfma(Ty, h(H0, 4, r + 1, x), h(H0, 4, r, x)), R(0.5)));
        o[5] = cadd(cscale(F[(5 * FR + fr) * N + x], n2), cscale(cfma(Tz, h(H1, 5, r, x), h(H0, 5, r, x)), R(0.5)));
        cx<R>* op = dst + zo * NN + (y0 + r) * N + x;
#pragma unroll
        for (int f = 0; f < 6; ++f) op[(long long)f * Nq] = o[f];
        if (wdot) {
          R a = 0;
#pragma unroll
          for (int f = 0; f < 6; ++f) {
            const cx<R> wf = F[(f * FR + fr) * N + x];
            a += wf.x * o[f].x + wf.y * o[f].y;
          }
          acc += double(a);
        }
      }
    }
  }
  if (wdot) {
    // one partial per CTA: [vec][blockIdx.y][blockIdx.x]
    __shared__ double red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid < 32) {
      double v = tid < (TPB + 31) / 32 ? red[tid] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (tid == 0)
        wdot[(long long)vec * gridDim.x * gridDim.y + blockIdx.y * gridDim.x + blockIdx.x] = make_double2(v, 0.0);
    }
  }
}

// Out of place: out = [M J^H; J N] w on 6-field vectors (stride 6*Nq).
// wdot (may be null): per-CTA partial sums of Re(w^H out), sweep_partials
// of them per vector.
template <class R, int N>
cudaError_t sweep_n(const Plan& P, const cx<R>* w, cx<R>* out, int nvec, const VecCtx& ctx, cudaStream_t st,
                    double2* wdot = nullptr) {
  using SH = SweepShape<R, N>;
  auto kfn = k_sweep<R, N>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SH::SMEM);
  if (e != cudaSuccess) return e;
  const dim3 g(N / SH::TY, N / SH::TZ, nvec);
  FAME_LAUNCHED(1);
  kfn<<<g, SH::TPB, SH::SMEM, st>>>(w, out, pdata<R>(P), P.d_phase, P.nphase, ctx, 6LL * N * N * N, wdot);
  return cudaGetLastError();
}

template <class R, int N> constexpr int sweep_partials_n() {
  return (N / SweepShape<R, N>::TY) * (N / SweepShape<R, N>::TZ);
}

// In place on w (6-field vectors, stride 6*Nq), scratch h of the same size;
// tpb threads per block of the two-kernel form (128, 256 or 512), or 0 for
// the single-pass k_sweep (through h, then copied back).
template <class R, int N>
cudaError_t stencil_n(const Plan& P, cx<R>* w, cx<R>* h, int nvec, const VecCtx& ctx, cudaStream_t st,
                      int tpb = 256) {
  constexpr int Nq = N * N * N;
  if (tpb == 0 && (((uintptr_t)w | (uintptr_t)h) & 15) == 0) {  // cp.async staging needs 16-byte rows
    cudaError_t e = sweep_n<R, N>(P, w, h, nvec, ctx, st);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(w, h, sizeof(cx<R>) * 6 * (size_t)Nq * nvec, cudaMemcpyDeviceToDevice, st);
  }
  if (tpb != 128 && tpb != 512) tpb = 256;
  const dim3 g((Nq + tpb - 1) / tpb, nvec);
  FAME_LAUNCHED(1);
  k_vertex<R, N><<<g, tpb, 0, st>>>(w, h, pdata<R>(P), P.d_phase, P.nphase, ctx, 6LL * Nq);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  FAME_LAUNCHED(1);
  k_faceedge<R, N><<<g, tpb, 0, st>>>(w, h, pdata<R>(P), P.d_phase, P.nphase, ctx, 6LL * Nq);
  return cudaGetLastError();
}

}  // namespace detail
}  // namespace fame
