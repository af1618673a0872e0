// Fused, TMA-pipelined RK stage of the FP32 shallow-water form (perturbation about the lake at rest).
//
// One persistent kernel per RK stage replaces the edge-flux + volume pair.  Each warp is an independent
// worker that owns one element at a time (N = 7: 64 nodes, two per lane) and walks over the elements
// e = warp, warp + total warps, ... with its own NBUF-deep pipeline: lanes of the warp issue 1-D TMA bulk
// copies (cp.async.bulk ... mbarrier::complete_tx) of the element blocks of a later element -- state q, RK
// register G, metrics, aux fields, lake-at-rest tendency, per-side edge data, its own and the neighbours'
// boundary traces -- into the warp's shared-memory buffers while the warp computes the current one.  No block-wide
// barrier is used after set-up; phases inside an element synchronise with __syncwarp.  Per element:
//   1. traces of the element's own state: staged with the element (the previous stage wrote them, by warp
//      shuffles over the registers of its node pairs, together with the new state);
//   2. LLF flux at the 32 side nodes (one per lane), evaluated exactly as the edge's primary element sees it
//      (primary trace "in", secondary trace "ex", primary normal and length), +flux on the primary side and
//      -flux on the secondary side, so both elements use bitwise-identical values as in EdgeFlux
//      (ConservativeShallowWaterClass.f90:1266-1360);
//   3. contravariant fluxes, the two weak-derivative contractions (each lane owns a node pair; derivative-matrix
//      rows held in registers, flux rows read as float4), lift, 1/J, sources, RK update;
//   4. new traces (shuffles) into the next trace buffer (three buffers rotate over the 3 stages of a step).
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
  int probe_polls;       // time-out test hook: polls of the first wait on a barrier nothing arrives on (0 = off)
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

// Square root and quotient on the special-function unit (rsqrt / reciprocal, 2 ulp): depths and gravity-wave
// speeds are positive, and the same inputs give the same outputs, so the lake-at-rest cancellation
// (fac = fac0 when eta = 0) stays exact.
__device__ __forceinline__ float sqrt_sfu(float x) { return x * rsqrtf(x); }
__device__ __forceinline__ float div_sfu(float a, float b) { return __fdividef(a, b); }

__device__ __forceinline__ void riemann_pert(const float* in, const float* ex, float hL, float hR, float nx, float ny,
                                             float g, float* f) {
  const float UL = in[0], VL = in[1], eL = in[2];
  const float UR = ex[0], VR = ex[1], eR = ex[2];
  const float pL = hL + eL, pR = hR + eR;
  const float uOut = UR * nx + VR * ny, uIn = UL * nx + VL * ny;
  const float wR = div_sfu(uOut, pR), wL = div_sfu(uIn, pL);
  const float cR = sqrt_sfu(g * pR), cL = sqrt_sfu(g * pL);
  const float fac = fmaxf(fmaxf(fabsf(wR + cR), fabsf(wR - cR)), fmaxf(fabsf(wL + cL), fabsf(wL - cL)));
  const float fac0 = fmaxf(sqrt_sfu(g * hR), sqrt_sfu(g * hL));
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
  float own[S::NB];  // the element's own traces (written by the previous stage), t = k + N1 v + 3 N1 side
};

template <int N1, int NBUF>
struct alignas(16) WarpSmem {
  WarpBuf<N1> buf[NBUF];
  ESide es[NBUF][4];
  float sB[4 * 3 * N1];  // side fluxes, same order
  uint64_t bar[NBUF];
  uint64_t probe;  // initialised, never arrived on: the wait of the time-out test hook runs out on it
  uint64_t pad[(NBUF + 1) & 1];
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

// Boundary traces of the 3-variable state held in registers (lane = node pair (i, j), (i + 1, j), i = 2 (lane % 4),
// j = lane / 4; N1 = 8), by warp shuffles.  S/N traces sum over j (lane bits 2-4), E/W traces over i (lane bits
// 0-1); each butterfly level splits the values still being summed between the two partners (reduce-scatter),
// so after the last level lane bit 4 selects S or N, bit 3 the node i or i + 1, and lane bit 0 selects E or W.
// The trace (side, v, k) is written at index k + N1 * v + 3 * N1 * side of `out` (shared or global memory).
__device__ __forceinline__ void traces_shfl(const float2 (&q)[3], float lSj, float lNj, float lEa, float lEb,
                                            float lWa, float lWb, int lane, int i, int j, float* out) {
  constexpr int N1 = 8;
  const bool b4 = lane & 16, b3 = lane & 8, b0 = lane & 1;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const float qa = q[v].x, qb = q[v].y;
    // S / N: sum over j
    const float sa = lSj * qa, sb = lSj * qb, na = lNj * qa, nb = lNj * qb;
    const float k0 = b4 ? na : sa, k1 = b4 ? nb : sb;
    const float x0 = k0 + __shfl_xor_sync(0xffffffffu, b4 ? sa : na, 16);
    const float x1 = k1 + __shfl_xor_sync(0xffffffffu, b4 ? sb : nb, 16);
    float y = (b3 ? x1 : x0) + __shfl_xor_sync(0xffffffffu, b3 ? x0 : x1, 8);
    y += __shfl_xor_sync(0xffffffffu, y, 4);
    if ((lane & 4) == 0) out[i + (b3 ? 1 : 0) + N1 * v + 3 * N1 * (b4 ? 2 : 0)] = y;
    // E / W: sum over i
    const float ev = lEa * qa + lEb * qb, wv = lWa * qa + lWb * qb;
    float z = (b0 ? wv : ev) + __shfl_xor_sync(0xffffffffu, b0 ? ev : wv, 1);
    z += __shfl_xor_sync(0xffffffffu, z, 2);
    if ((lane & 2) == 0) out[j + N1 * v + 3 * N1 * (b0 ? 3 : 1)] = z;
  }
}

// Lane map (N1 = 8): lane owns the node pair (i, j), (i + 1, j) with i = 2 (lane % 4), j = lane / 4, i.e. the
// flat nodes 2 lane and 2 lane + 1, so every per-node field moves as a float2.
// MODE 1: G = tendency (first RK stage), 2: G = a G + tendency; EXTRA: linear drag and/or relaxation present.
template <int N1, int NBUF, int W, int MODE, bool EXTRA>
__global__ void __launch_bounds__(32 * W, 4) sw32_fused(FusedArgs A, FConst<N1> Cg) {
  constexpr int NN = N1 * N1;
  static_assert(N1 == 8, "fused stage: lane map (node pairs, 32 side nodes) and 16-byte bulk granularity");
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
    mbar_init(&ws.probe, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();  // the only block-wide barrier: constants and barrier initialisation
  const FConst<N1>& C = sm.C;
  const int i = 2 * (lane & 3), j = lane >> 2;
  const int node = 2 * lane;  // = i + N1 * j
  float cS0[N1], cS1[N1];
#pragma unroll
  for (int m = 0; m < N1; ++m) {
    cS0[m] = C.dS[i + N1 * m];
    cS1[m] = C.dS[i + 1 + N1 * m];
  }
  const float lEa = C.lE[i], lWa = C.lW[i], qwa = C.qwinv[i];
  const float lEb = C.lE[i + 1], lWb = C.lW[i + 1], qwb = C.qwinv[i + 1];
  const float lNj = C.lN[j], lSj = C.lS[j], qwj = C.qwinv[j];

  // Programmatic dependent launch: the next stage's CTAs may be scheduled as this grid's CTAs retire, and this
  // grid's set-up overlaps the previous stage's tail; every read or write of data the previous stage touches
  // (state, RK register, traces) comes after the wait for that stage's completion (griddepcontrol.wait below).
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int nwarps = gridDim.x * W;
  const int gw = blockIdx.x * W + wid;
  const long long kMaxSpin = 1LL << 20;  // try_wait polls; normal waits end within microseconds
  const uint32_t base_bytes =
      4u * (S::Q + S::M + (uint32_t)A.naux * NN + S::R + S::EG + S::NB) + (MODE == 2 ? 4u * S::G : 0u);

  // issue the bulk copies of element e into buffer b: lanes 0-3 the neighbour traces of side = lane, lanes
  // 4-10 the element blocks; the byte count is posted before any copy is issued.  part 1 posts the count and
  // copies only the blocks no stage writes (metrics, aux, R0, side geometry), part 2 the rest (state, RK
  // register, traces), part 0 everything.
  // side records of element e (lanes 0-3), loaded one iteration before the element's copies are issued
  auto load_es = [&](int e) {
    ESide es;
    es.nbr = -1;
    if (lane < 4 && e < A.nEl) es = A.es[e * 4 + lane];
    return es;
  };
  auto issue = [&](int e, int b, const ESide& es, int part) {
    const bool hasnb = lane < 4 && es.nbr >= 0;
    if (part != 2) {
      if (lane < 4) ws.es[b][lane] = es;
      const unsigned nbm = __ballot_sync(0xffffffffu, hasnb);
      fence_proxy_async();  // earlier generic accesses of this buffer before the async-proxy writes
      __syncwarp();
      if (lane == 0) mbar_expect_tx(&ws.bar[b], base_bytes + (uint32_t)__popc(nbm) * 4u * 3u * N1);
      __syncwarp();
    }
    WarpBuf<N1>& B = ws.buf[b];
    const bool stat = part != 2, dyn = part != 1;
    if (hasnb) {
      if (dyn)
        bulk_g2s(&B.nb[lane * 3 * N1], A.bs_in + 3 * N1 * (es.nside + 4 * es.nbr), 4u * 3u * N1, &ws.bar[b]);
    } else if (lane == 4) {
      if (dyn) bulk_g2s(B.q, A.q + e * S::Q, 4u * S::Q, &ws.bar[b]);
    } else if (lane == 5) {
      if (stat) bulk_g2s(B.met, A.met + e * S::M, 4u * S::M, &ws.bar[b]);
    } else if (lane == 6) {
      if (stat) bulk_g2s(B.aux, A.aux + e * A.naux * NN, 4u * A.naux * NN, &ws.bar[b]);
    } else if (lane == 7) {
      if (stat) bulk_g2s(B.R0, A.R0 + e * S::R, 4u * S::R, &ws.bar[b]);
    } else if (lane == 8) {
      if (stat) bulk_g2s(B.eg, A.eg + e * S::EG, 4u * S::EG, &ws.bar[b]);
    } else if (lane == 10) {
      if (dyn) bulk_g2s(B.own, A.bs_in + e * S::NB, 4u * S::NB, &ws.bar[b]);
    } else if (MODE == 2 && lane == 9) {
      if (dyn) bulk_g2s(B.G, A.G + e * S::G, 4u * S::G, &ws.bar[b]);
    }
  };

  // prologue: elements of iterations 0 .. NBUF-2; their blocks that no stage writes are requested before the
  // wait for the previous stage (they overlap its tail), the others after it
  ESide es_pro[NBUF > 1 ? NBUF - 1 : 1];
#pragma unroll
  for (int k = 0; k < NBUF - 1; ++k) {
    const int e = gw + k * nwarps;
    es_pro[k] = load_es(e);
    if (e < A.nEl) issue(e, k, es_pro[k], 1);
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
#pragma unroll
  for (int k = 0; k < NBUF - 1; ++k) {
    const int e = gw + k * nwarps;
    if (e < A.nEl) issue(e, k, es_pro[k], 2);
  }
  ESide es_next = load_es(gw + (NBUF - 1) * nwarps);
  int it = 0;
  for (int e = gw; e < A.nEl; e += nwarps, ++it) {
    const int b = it % NBUF;
    {
      const int ef = e + (NBUF - 1) * nwarps;  // buffer (b + NBUF - 1) % NBUF was released by iteration it - 1
      if (ef < A.nEl) {
        issue(ef, (b + NBUF - 1) % NBUF, es_next, 0);
        es_next = load_es(ef + nwarps);
      }
    }
    // time-out test hook (0 in normal runs): the first wait of every warp polls a barrier nothing arrives on, runs
    // out after A.probe_polls polls and takes the time-out path below
    const bool ok = (A.probe_polls > 0 && it == 0) ? mbar_wait(&ws.probe, 0u, A.probe_polls)
                                                   : mbar_wait(&ws.bar[b], (uint32_t)((it / NBUF) & 1), kMaxSpin);
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
    // registers: state, metrics and bathymetry of the node pair
    float2 q2[3], m2[5];
#pragma unroll
    for (int v = 0; v < 3; ++v) q2[v] = *reinterpret_cast<const float2*>(&B.q[v * NN + node]);
#pragma unroll
    for (int c = 0; c < 5; ++c) m2[c] = *reinterpret_cast<const float2*>(&B.met[c * NN + node]);
    const float2 h2 = *reinterpret_cast<const float2*>(&B.aux[3 * NN + node]);
    // 1. own traces: the previous stage wrote them with the new state (staged with the element)
    __syncwarp();  // q and met are free (scratch)
    float* sF = B.q;            // [3][NN], natural order
    float* sGt = B.q + 3 * NN;  // [3][N1 rows of 12]: sGt[v][m + 12 i] = G_v(i, m)
    // 2. side fluxes: lane = (side, k)
    {
      const int side = lane >> 3, k = lane & 7;
      const ESide es = ws.es[b][side];
      const int flags = es.b_flags & 0xff, bb = es.b_flags >> 8;
      const float* egs = &B.eg[side * 5 * N1];
      const float nx = egs[k], ny = egs[N1 + k], len = egs[2 * N1 + k], hP = egs[3 * N1 + k], hS = egs[4 * N1 + k];
      float own[3], oth[3], in[3], ex[3], f[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) own[v] = B.own[k + N1 * v + 3 * N1 * side];
      // one flux evaluation for every lane (no divergence between the interior-primary, interior-secondary and
      // wall sides of the warp): the external state and the orientation are selected, hS = hP on walls.
      // A wall side has a = 0, b = 1, so kn stays a valid index; its neighbour slot is not read into the flux.
      const bool interior = es.nbr >= 0;
      const bool primary = !interior || (flags & 1);
      const int kn = es.a + bb * k;
      const float mirror0 = (ny * ny - nx * nx) * own[0] - 2.0f * nx * ny * own[1];  // NO_NORMAL_FLOW
      const float mirror1 = (nx * nx - ny * ny) * own[1] - 2.0f * nx * ny * own[0];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const float nbv = B.nb[side * 3 * N1 + v * N1 + kn];
        oth[v] = interior ? nbv : (v == 0 ? mirror0 : v == 1 ? mirror1 : own[2]);
        in[v] = primary ? own[v] : oth[v];
        ex[v] = primary ? oth[v] : own[v];
      }
      riemann_pert(in, ex, hP, hS, nx, ny, A.g, f);
      const float sgn = primary ? 1.f : -1.f;
#pragma unroll
      for (int v = 0; v < 3; ++v) ws.sB[k + N1 * v + 3 * N1 * side] = sgn * (f[v] * len);
    }
    // 3. contravariant fluxes of the node pair
    {
      auto cflux = [&](float U, float V, float eta, float hn, float dxds, float dxdp, float dyds, float dydp,
                       float* Ft, float* Gt) {
        const float iH = div_sfu(1.0f, hn + eta);
        const float p = A.g * eta * (hn + 0.5f * eta);
        float xF[3], yF[3];
        xF[0] = U * U * iH + p;
        xF[1] = U * V * iH;
        xF[2] = U;
        yF[0] = V * U * iH;
        yF[1] = V * V * iH + p;
        yF[2] = V;
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          Ft[v] = dydp * xF[v] - dxdp * yF[v];
          Gt[v] = -dyds * xF[v] + dxds * yF[v];
        }
      };
      float Fa[3], Ga[3], Fb[3], Gb[3];
      cflux(q2[0].x, q2[1].x, q2[2].x, h2.x, m2[0].x, m2[1].x, m2[2].x, m2[3].x, Fa, Ga);
      cflux(q2[0].y, q2[1].y, q2[2].y, h2.y, m2[0].y, m2[1].y, m2[2].y, m2[3].y, Fb, Gb);
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        *reinterpret_cast<float2*>(&sF[v * NN + node]) = make_float2(Fa[v], Fb[v]);
        sGt[v * 12 * N1 + j + 12 * i] = Ga[v];
        sGt[v * 12 * N1 + j + 12 * (i + 1)] = Gb[v];
      }
    }
    __syncwarp();
    // 4. contractions, lift, sources, RK update
    const float4 cPa = reinterpret_cast<const float4*>(&C.dPt[N1 * j])[0];  // dP[j + N1 m], m = 0..7
    const float4 cPb = reinterpret_cast<const float4*>(&C.dPt[N1 * j])[1];
    const float cP[N1] = {cPa.x, cPa.y, cPa.z, cPa.w, cPb.x, cPb.y, cPb.z, cPb.w};
    float2 tend[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      const float4* Fr = reinterpret_cast<const float4*>(&sF[v * NN + N1 * j]);
      const float4* Ga4 = reinterpret_cast<const float4*>(&sGt[v * 12 * N1 + 12 * i]);
      const float4* Gb4 = reinterpret_cast<const float4*>(&sGt[v * 12 * N1 + 12 * (i + 1)]);
      const float4 f0 = Fr[0], f1 = Fr[1];
      const float4 ga0 = Ga4[0], ga1 = Ga4[1], gb0 = Gb4[0], gb1 = Gb4[1];
      float dsa = 0.f, dsb = 0.f, dpa = 0.f, dpb = 0.f;
      dsa += cS0[0] * f0.x; dsa += cS0[1] * f0.y; dsa += cS0[2] * f0.z; dsa += cS0[3] * f0.w;
      dsa += cS0[4] * f1.x; dsa += cS0[5] * f1.y; dsa += cS0[6] * f1.z; dsa += cS0[7] * f1.w;
      dsb += cS1[0] * f0.x; dsb += cS1[1] * f0.y; dsb += cS1[2] * f0.z; dsb += cS1[3] * f0.w;
      dsb += cS1[4] * f1.x; dsb += cS1[5] * f1.y; dsb += cS1[6] * f1.z; dsb += cS1[7] * f1.w;
      const float bE = ws.sB[j + N1 * v + 3 * N1 * 1], bW = ws.sB[j + N1 * v + 3 * N1 * 3];
      dsa += (bE * lEa + bW * lWa) * qwa;
      dsb += (bE * lEb + bW * lWb) * qwb;
      dpa += cP[0] * ga0.x; dpa += cP[1] * ga0.y; dpa += cP[2] * ga0.z; dpa += cP[3] * ga0.w;
      dpa += cP[4] * ga1.x; dpa += cP[5] * ga1.y; dpa += cP[6] * ga1.z; dpa += cP[7] * ga1.w;
      dpb += cP[0] * gb0.x; dpb += cP[1] * gb0.y; dpb += cP[2] * gb0.z; dpb += cP[3] * gb0.w;
      dpb += cP[4] * gb1.x; dpb += cP[5] * gb1.y; dpb += cP[6] * gb1.z; dpb += cP[7] * gb1.w;
      const float2 bN = *reinterpret_cast<const float2*>(&ws.sB[i + N1 * v + 3 * N1 * 2]);
      const float2 bS = *reinterpret_cast<const float2*>(&ws.sB[i + N1 * v + 3 * N1 * 0]);
      dpa += (bN.x * lNj + bS.x * lSj) * qwj;
      dpb += (bN.y * lNj + bS.y * lSj) * qwj;
      tend[v].x = (-dsa - dpa) * m2[4].x;
      tend[v].y = (-dsb - dpb) * m2[4].y;
    }
    {
      const float2 dhdx = *reinterpret_cast<const float2*>(&B.aux[node]);
      const float2 dhdy = *reinterpret_cast<const float2*>(&B.aux[NN + node]);
      const float2 fc = *reinterpret_cast<const float2*>(&B.aux[2 * NN + node]);
      auto source = [&](float U, float V, float eta, float hn, float dx, float dy, float f, float ts, float* s) {
        s[0] = f * V + A.g * eta * dx;
        s[1] = -f * U + A.g * eta * dy;
        s[2] = 0.f;
        if (EXTRA && A.has_drag) {
          s[0] -= A.drag * U / hn;
          s[1] -= A.drag * V / hn;
        }
        if (EXTRA && A.has_relax) {
          s[0] -= U * ts;
          s[1] -= V * ts;
          s[2] -= eta * ts;
        }
      };
      float2 ts2 = make_float2(0.f, 0.f);
      if (EXTRA && A.has_relax) ts2 = *reinterpret_cast<const float2*>(&B.aux[4 * NN + node]);
      float sa[3], sb[3];
      source(q2[0].x, q2[1].x, q2[2].x, h2.x, dhdx.x, dhdy.x, fc.x, ts2.x, sa);
      source(q2[0].y, q2[1].y, q2[2].y, h2.y, dhdx.y, dhdy.y, fc.y, ts2.y, sb);
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const float2 r0 = *reinterpret_cast<const float2*>(&B.R0[v * NN + node]);
        tend[v].x += sa[v] + r0.x;
        tend[v].y += sb[v] + r0.y;
      }
    }
    float2* Ge = reinterpret_cast<float2*>(A.G + e * 3 * NN);
    float2* qo = reinterpret_cast<float2*>(A.qout + e * 3 * NN);
    float2 qn[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      float2 gg = tend[v];
      if (MODE == 2) {
        const float2 g0 = *reinterpret_cast<const float2*>(&B.G[v * NN + node]);
        gg.x = A.a * g0.x + tend[v].x;
        gg.y = A.a * g0.y + tend[v].y;
      }
      Ge[(v * NN + node) / 2] = gg;
      qn[v].x = q2[v].x + A.gdt * gg.x;
      qn[v].y = q2[v].y + A.gdt * gg.y;
      qo[(v * NN + node) / 2] = qn[v];
    }
    // 5. traces of the new state
    traces_shfl(qn, lSj, lNj, lEa, lEb, lWa, lWb, lane, i, j, A.bs_out + 3 * N1 * 4 * e);
    __syncwarp();  // this buffer's floats are read; the next issue into it follows a proxy fence
  }
}

}  // namespace sw32
}  // namespace selfgpu
