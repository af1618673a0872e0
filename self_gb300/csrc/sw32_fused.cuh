// Fused, TMA-pipelined RK stage of the FP32 shallow-water form (perturbation about the lake at rest).
//
// One persistent kernel per RK stage replaces the edge-flux + volume pair.  Each warp is an independent
// worker that owns one element at a time (N = 7: 64 nodes, two per lane) and walks over the elements
// e = warp, warp + total warps, ... with its own NBUF-deep pipeline: lanes of the warp issue 1-D TMA bulk
// copies (cp.async.bulk ... mbarrier::complete_tx) of the element blocks of a later element -- state q, RK
// register G, metrics, aux fields, lake-at-rest tendency, per-side edge data and the neighbours' boundary
// traces -- into the warp's shared-memory buffers while the warp computes the current one.  No block-wide
// barrier is used after set-up; phases inside an element synchronise with __syncwarp.  Per element:
//   1. traces of the element's own state (shared memory, 3 values per lane);
//   2. LLF flux at the 32 side nodes (one per lane), evaluated exactly as the edge's primary element sees it
//      (primary trace "in", secondary trace "ex", primary normal and length), +flux on the primary side and
//      -flux on the secondary side, so both elements use bitwise-identical values as in EdgeFlux
//      (ConservativeShallowWaterClass.f90:1266-1360);
//   3. contravariant fluxes, the two weak-derivative contractions (derivative-matrix rows held in registers,
//      flux rows read as float4), lift, 1/J, sources, RK update;
//   4. new traces into the next trace buffer (three buffers rotate over the 3 stages of a step).
// Every mbarrier wait is bounded; on time-out the warp records an error code, drains its own copies with a
// second bounded wait and returns (the host reports SELF_ERR_TIMEOUT).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace selfgpu {
namespace sw32 {

// per element side: neighbour element (0-based, -1 = boundary), neighbour side, neighbour index map
// nbr_node = a + b * own_node, flags (bit 0: this element is the edge's primary; bit 1: boundary wall)
struct ESide {
  int nbr, nside, a, b_flags;  // b_flags: b (+1/-1) in bits 8.., flags in bits 0..7
};

struct FusedArgs {
  const float* q;        // [nEl][3][NN]
  float* qout;           // may alias q (each element touched by its own CTA only)
  float* G;              // [nEl][3][NN]
  const float* met;      // [nEl][5][NN]  dxds, dxdp, dyds, dydp, 1/J
  const float* aux;      // [nEl][naux][NN] dhdx, dhdy, f, h [, ts]
  const float* R0;       // [nEl][3][NN]
  const float* eg;       // [nEl][4][5][N1] nx, ny, len (primary's), hP, hS
  const ESide* es;       // [nEl][4]
  const float* bs_in;    // traces of the current state [nEl][4][3][N1]
  float* bs_out;         // traces of the new state
  int* err;              // error flag (time-out)
  int nEl, naux, has_drag, has_relax, mode;  // mode 1: G = tend, 2: G = a G + tend
  float g, drag, a, gdt;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bounded wait for the phase with the given parity; returns false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long max_iters) {
  uint32_t done = 0;
  for (long long it = 0; it < max_iters; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 1-D TMA bulk copy global -> shared, completion on the mbarrier (sizes and addresses multiples of 16 bytes)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <int N1>
struct FConst {
  float dS[N1 * N1], dP[N1 * N1];
  float dPt[N1 * N1];  // dPt[j * N1 + m] = dP[j + N1 * m] (rows read as float4)
  float lW[N1], lE[N1], lS[N1], lN[N1];
  float qwinv[N1];
};

__device__ __forceinline__ void riemann_pert(const float* in, const float* ex, float hL, float hR, float nx, float ny,
                                             float g, float* f) {
  const float UL = in[0], VL = in[1], eL = in[2];
  const float UR = ex[0], VR = ex[1], eR = ex[2];
  const float pL = hL + eL, pR = hR + eR;
  const float uOut = UR * nx + VR * ny, uIn = UL * nx + VL * ny;
  const float wR = uOut / pR, wL = uIn / pL;
  const float cR = sqrtf(g * pR), cL = sqrtf(g * pL);
  const float fac = fmaxf(fmaxf(fabsf(wR + cR), fabsf(wR - cR)), fmaxf(fabsf(wL + cL), fabsf(wL - cL)));
  const float fac0 = fmaxf(sqrtf(g * hR), sqrtf(g * hL));
  const float pr = 0.5f * g * eR * (2.0f * hR + eR), pl = 0.5f * g * eL * (2.0f * hL + eL);
  f[0] = 0.5f * ((wR * UR + pr * nx + wL * UL + pl * nx) - fac * (UR - UL));
  f[1] = 0.5f * ((wR * VR + pr * ny + wL * VL + pl * ny) - fac * (VR - VL));
  f[2] = 0.5f * ((uOut + uIn) - fac * (eR - eL) - (fac - fac0) * (hR - hL));
}

template <int N1>
struct WarpStage {  // floats staged per element, one block per field (all multiples of 16 bytes for N1 = 8)
  static constexpr int NN = N1 * N1;
  static constexpr int Q = 3 * NN, M = 5 * NN, G = 3 * NN, AUX = 5 * NN, R = 3 * NN, EG = 4 * 5 * N1,
                       NB = 4 * 3 * N1;
};

// One element's staging buffer.  q and met are adjacent: once their values are in registers the 8 * NN floats
// are reused as scratch (contravariant fluxes F in natural order, G transposed with a padded row of 12 floats,
// then the new state).
template <int N1>
struct alignas(16) WarpBuf {
  using S = WarpStage<N1>;
  float q[S::Q];
  float met[S::M];
  float G[S::G];
  float aux[S::AUX];
  float R0[S::R];
  float eg[S::EG];
  float nb[S::NB];  // neighbour traces per side (the neighbour's side, neighbour node order)
};

template <int N1, int NBUF>
struct alignas(16) WarpSmem {
  WarpBuf<N1> buf[NBUF];
  ESide es[NBUF][4];
  float sT[4 * 3 * N1];  // own traces, t = k + N1 * v + 3 * N1 * side
  float sB[4 * 3 * N1];  // side fluxes, same order
  uint64_t bar[NBUF];
  uint64_t pad[NBUF & 1];
};

template <int N1, int NBUF, int W>
struct FusedSmem {
  WarpSmem<N1, NBUF> w[W];
  FConst<N1> C;
};

template <int N1, int NBUF, int W>
constexpr size_t fused_smem_bytes() {
  return sizeof(FusedSmem<N1, NBUF, W>);
}

// trace value t = k + N1 * v + 3 * N1 * side of the 3-variable state Q[v * NN + i + N1 * j]
template <int N1>
__device__ __forceinline__ float trace_value(const float* Q, const FConst<N1>& C, int t) {
  constexpr int NN = N1 * N1;
  const int k = t % N1, v = (t / N1) % 3, side = t / (3 * N1);
  const float* L = (side == 0) ? C.lS : (side == 1) ? C.lE : (side == 2) ? C.lN : C.lW;
  const int base = v * NN + ((side & 1) ? N1 * k : k);
  const int stride = (side & 1) ? 1 : N1;
  float acc = 0.f;
#pragma unroll
  for (int m = 0; m < N1; ++m) acc += L[m] * Q[base + stride * m];
  return acc;
}

// NBUF = 2 with W = 4 fits 16 warps per SM (128 registers, 51 KB of shared memory per CTA); NBUF = 3 with W = 3
// fits 12 warps (55 KB per CTA)
template <int N1, int NBUF, int W>
__global__ void __launch_bounds__(32 * W, 4) sw32_fused(FusedArgs A, FConst<N1> Cg) {
  constexpr int NN = N1 * N1;
  static_assert(N1 == 8, "fused stage: lane map (2 nodes per lane, 32 side nodes) and 16-byte bulk granularity");
  using S = WarpStage<N1>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  FusedSmem<N1, NBUF, W>& sm = *reinterpret_cast<FusedSmem<N1, NBUF, W>*>(smem_raw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  WarpSmem<N1, NBUF>& ws = sm.w[wid];
  {
    constexpr int NC = sizeof(FConst<N1>) / sizeof(float);
    const float* src = reinterpret_cast<const float*>(&Cg);
    float* dst = reinterpret_cast<float*>(&sm.C);
    for (int t = threadIdx.x; t < NC; t += 32 * W) dst[t] = src[t];
  }
  if (lane == 0) {
    for (int b = 0; b < NBUF; ++b) mbar_init(&ws.bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();  // the only block-wide barrier: constants and barrier initialisation
  const FConst<N1>& C = sm.C;
  const int i = lane & 7, j = lane >> 3;  // nodes (i, j) and (i, j + 4)
  float cS[N1];
#pragma unroll
  for (int m = 0; m < N1; ++m) cS[m] = C.dS[i + N1 * m];
  const float lEi = C.lE[i], lWi = C.lW[i], qwi = C.qwinv[i];
  const float lN0 = C.lN[j], lS0 = C.lS[j], qw0 = C.qwinv[j];
  const float lN1 = C.lN[j + 4], lS1 = C.lS[j + 4], qw1 = C.qwinv[j + 4];

  const int nwarps = gridDim.x * W;
  const int gw = blockIdx.x * W + wid;
  const long long kMaxSpin = 1LL << 20;  // try_wait polls; normal waits end within microseconds
  const uint32_t base_bytes = 4u * (S::Q + S::M + (uint32_t)A.naux * NN + S::R + S::EG) + (A.mode == 2 ? 4u * S::G : 0u);

  // issue the bulk copies of element e into buffer b: lanes 0-3 the neighbour traces of side = lane, lanes
  // 4-9 the element blocks; the byte count is posted before any copy is issued
  auto issue = [&](int e, int b) {
    ESide es;
    es.nbr = -1;
    if (lane < 4) {
      es = A.es[(size_t)e * 4 + lane];
      ws.es[b][lane] = es;
    }
    const bool hasnb = lane < 4 && es.nbr >= 0;
    const unsigned nbm = __ballot_sync(0xffffffffu, hasnb);
    fence_proxy_async();  // earlier generic accesses of this buffer before the async-proxy writes
    __syncwarp();
    if (lane == 0) mbar_expect_tx(&ws.bar[b], base_bytes + (uint32_t)__popc(nbm) * 4u * 3u * N1);
    __syncwarp();
    WarpBuf<N1>& B = ws.buf[b];
    if (hasnb)
      bulk_g2s(&B.nb[lane * 3 * N1], A.bs_in + (size_t)3 * N1 * (es.nside + 4 * (size_t)es.nbr), 4u * 3u * N1,
               &ws.bar[b]);
    else if (lane == 4)
      bulk_g2s(B.q, A.q + (size_t)e * S::Q, 4u * S::Q, &ws.bar[b]);
    else if (lane == 5)
      bulk_g2s(B.met, A.met + (size_t)e * S::M, 4u * S::M, &ws.bar[b]);
    else if (lane == 6)
      bulk_g2s(B.aux, A.aux + (size_t)e * A.naux * NN, 4u * A.naux * NN, &ws.bar[b]);
    else if (lane == 7)
      bulk_g2s(B.R0, A.R0 + (size_t)e * S::R, 4u * S::R, &ws.bar[b]);
    else if (lane == 8)
      bulk_g2s(B.eg, A.eg + (size_t)e * S::EG, 4u * S::EG, &ws.bar[b]);
    else if (lane == 9 && A.mode == 2)
      bulk_g2s(B.G, A.G + (size_t)e * S::G, 4u * S::G, &ws.bar[b]);
  };

  // prologue: elements of iterations 0 .. NBUF-2
#pragma unroll
  for (int k = 0; k < NBUF - 1; ++k) {
    const int e = gw + k * nwarps;
    if (e < A.nEl) issue(e, k);
  }
  int it = 0;
  for (int e = gw; e < A.nEl; e += nwarps, ++it) {
    const int b = it % NBUF;
    {
      const int ef = e + (NBUF - 1) * nwarps;  // buffer (b + NBUF - 1) % NBUF was released by iteration it - 1
      if (ef < A.nEl) issue(ef, (b + NBUF - 1) % NBUF);
    }
    const bool ok = mbar_wait(&ws.bar[b], (uint32_t)((it / NBUF) & 1), kMaxSpin);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) atomicExch(A.err, 1);
      // drain: a second bounded wait on every buffer with copies in flight, then leave
      for (int k = 0; k < NBUF; ++k) {
        const int ek = e + k * nwarps;
        if (ek < A.nEl) mbar_wait(&ws.bar[(it + k) % NBUF], (uint32_t)(((it + k) / NBUF) & 1), kMaxSpin);
      }
      return;
    }
    WarpBuf<N1>& B = ws.buf[b];
    // registers: state and metrics of the two nodes
    float q0[3], q1[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      q0[v] = B.q[v * NN + lane];
      q1[v] = B.q[v * NN + lane + 32];
    }
    float m0[5], m1[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      m0[c] = B.met[c * NN + lane];
      m1[c] = B.met[c * NN + lane + 32];
    }
    const float h0 = B.aux[3 * NN + lane], h1 = B.aux[3 * NN + lane + 32];
    // 1. own traces
#pragma unroll
    for (int r = 0; r < 3; ++r) ws.sT[lane + 32 * r] = trace_value<N1>(B.q, C, lane + 32 * r);
    __syncwarp();  // q and met are free (scratch) and the own traces are visible
    float* sF = B.q;             // [3][NN], natural order
    float* sGt = B.q + 3 * NN;   // [3][N1 rows of 12]: sGt[v][m + 12 i] = G_v(i, m)
    // 2. side fluxes: lane = (side, k)
    {
      const int side = lane >> 3, k = lane & 7;
      const ESide es = ws.es[b][side];
      const int flags = es.b_flags & 0xff, bb = es.b_flags >> 8;
      const float* egs = &B.eg[side * 5 * N1];
      const float nx = egs[k], ny = egs[N1 + k], len = egs[2 * N1 + k], hP = egs[3 * N1 + k], hS = egs[4 * N1 + k];
      float own[3], oth[3], f[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) own[v] = ws.sT[k + N1 * v + 3 * N1 * side];
      float sgn = 1.f;
      if (es.nbr >= 0) {
        const int kn = es.a + bb * k;
#pragma unroll
        for (int v = 0; v < 3; ++v) oth[v] = B.nb[side * 3 * N1 + v * N1 + kn];
        if (flags & 1) {
          riemann_pert(own, oth, hP, hS, nx, ny, A.g, f);
        } else {
          riemann_pert(oth, own, hP, hS, nx, ny, A.g, f);
          sgn = -1.f;
        }
      } else {
        oth[0] = (ny * ny - nx * nx) * own[0] - 2.0f * nx * ny * own[1];  // mirror (NO_NORMAL_FLOW)
        oth[1] = (nx * nx - ny * ny) * own[1] - 2.0f * nx * ny * own[0];
        oth[2] = own[2];
        riemann_pert(own, oth, hP, hP, nx, ny, A.g, f);
      }
#pragma unroll
      for (int v = 0; v < 3; ++v) ws.sB[k + N1 * v + 3 * N1 * side] = sgn * (f[v] * len);
    }
    // 3. contravariant fluxes of the two nodes
    {
      auto cflux = [&](const float* qv, const float* me, float hn, int node, int ii, int jj) {
        const float iH = 1.0f / (hn + qv[2]);
        const float p = A.g * qv[2] * (hn + 0.5f * qv[2]);
        float xF[3], yF[3];
        xF[0] = qv[0] * qv[0] * iH + p;
        xF[1] = qv[0] * qv[1] * iH;
        xF[2] = qv[0];
        yF[0] = qv[1] * qv[0] * iH;
        yF[1] = qv[1] * qv[1] * iH + p;
        yF[2] = qv[1];
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          sF[v * NN + node] = me[3] * xF[v] - me[1] * yF[v];           // dydp xF - dxdp yF
          sGt[v * 12 * N1 + jj + 12 * ii] = -me[2] * xF[v] + me[0] * yF[v];  // -dyds xF + dxds yF
        }
      };
      cflux(q0, m0, h0, lane, i, j);
      cflux(q1, m1, h1, lane + 32, i, j + 4);
    }
    __syncwarp();
    // 4. contractions, lift, sources, RK update
    float* Ge = A.G + (size_t)e * 3 * NN;
    float* qo = A.qout + (size_t)e * 3 * NN;
    const float* ae = B.aux;
    float qn0[3], qn1[3];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int jj = j + 4 * half, node = lane + 32 * half;
      const float4 cpa = reinterpret_cast<const float4*>(&C.dPt[N1 * jj])[0];
      const float4 cpb = reinterpret_cast<const float4*>(&C.dPt[N1 * jj])[1];
      const float lN = half ? lN1 : lN0, lS = half ? lS1 : lS0, qwj = half ? qw1 : qw0;
      const float* qv = half ? q1 : q0;
      const float invJ = half ? m1[4] : m0[4];
      const float hn = half ? h1 : h0;
      float tend[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const float4* Fr = reinterpret_cast<const float4*>(&sF[v * NN + N1 * jj]);
        const float4* Gr = reinterpret_cast<const float4*>(&sGt[v * 12 * N1 + 12 * i]);
        const float4 f0 = Fr[0], f1 = Fr[1], g0 = Gr[0], g1 = Gr[1];
        float ds = 0.f, dp = 0.f;
        ds += cS[0] * f0.x; ds += cS[1] * f0.y; ds += cS[2] * f0.z; ds += cS[3] * f0.w;
        ds += cS[4] * f1.x; ds += cS[5] * f1.y; ds += cS[6] * f1.z; ds += cS[7] * f1.w;
        ds += (ws.sB[jj + N1 * v + 3 * N1 * 1] * lEi + ws.sB[jj + N1 * v + 3 * N1 * 3] * lWi) * qwi;
        dp += cpa.x * g0.x; dp += cpa.y * g0.y; dp += cpa.z * g0.z; dp += cpa.w * g0.w;
        dp += cpb.x * g1.x; dp += cpb.y * g1.y; dp += cpb.z * g1.z; dp += cpb.w * g1.w;
        dp += (ws.sB[i + N1 * v + 3 * N1 * 2] * lN + ws.sB[i + N1 * v + 3 * N1 * 0] * lS) * qwj;
        tend[v] = (-ds - dp) * invJ;
      }
      const float dhdx = ae[node], dhdy = ae[NN + node], fc = ae[2 * NN + node];
      float s0 = fc * qv[1] + A.g * qv[2] * dhdx;
      float s1 = -fc * qv[0] + A.g * qv[2] * dhdy;
      float s2 = 0.f;
      if (A.has_drag) {
        s0 -= A.drag * qv[0] / hn;
        s1 -= A.drag * qv[1] / hn;
      }
      if (A.has_relax) {
        const float ts = ae[4 * NN + node];
        s0 -= qv[0] * ts;
        s1 -= qv[1] * ts;
        s2 -= qv[2] * ts;
      }
      tend[0] += s0 + B.R0[node];
      tend[1] += s1 + B.R0[NN + node];
      tend[2] += s2 + B.R0[2 * NN + node];
      float* qn = half ? qn1 : qn0;
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const float gg = (A.mode == 2) ? (A.a * B.G[v * NN + node] + tend[v]) : tend[v];
        Ge[v * NN + node] = gg;
        qn[v] = qv[v] + A.gdt * gg;
        qo[v * NN + node] = qn[v];
      }
    }
    __syncwarp();  // scratch reads done: the new state goes into the same floats
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      sF[v * NN + lane] = qn0[v];
      sF[v * NN + lane + 32] = qn1[v];
    }
    __syncwarp();
    // 5. traces of the new state
    float* bo = A.bs_out + (size_t)3 * N1 * 4 * e;
#pragma unroll
    for (int r = 0; r < 3; ++r) bo[lane + 32 * r] = trace_value<N1>(sF, C, lane + 32 * r);
    __syncwarp();  // this buffer's floats are read; the next issue into it follows a proxy fence
  }
}

}  // namespace sw32
}  // namespace selfgpu
