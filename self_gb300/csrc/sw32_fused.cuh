// Fused, TMA-pipelined RK stage of the FP32 shallow-water form (perturbation about the lake at rest).
//
// One persistent kernel per RK stage replaces the edge-flux + volume pair.  Each CTA owns EPB elements at a
// time (64 threads per element at N = 7) and walks over element chunks with a two-deep pipeline: warp 0
// issues 1-D TMA bulk copies (cp.async.bulk ... mbarrier::complete_tx) of the next chunk's element-contiguous
// blocks -- state q, RK register G, metrics, aux fields, lake-at-rest tendency, per-side edge data and the
// neighbours' boundary traces -- into shared memory while the CTA computes the current chunk.  Per chunk:
//   1. traces of the element's own state (from shared memory);
//   2. LLF flux on each of its 4 sides, evaluated exactly as the edge's primary element sees it (primary trace
//      "in", secondary trace "ex", primary normal and length), +flux on the primary side and -flux on the
//      secondary side, so both elements use bitwise-identical values as in EdgeFlux
//      (ConservativeShallowWaterClass.f90:1266-1360);
//   3. contravariant fluxes, the two weak-derivative contractions, lift, 1/J, sources, RK update;
//   4. new traces into the next trace buffer (three buffers rotate over the 3 stages of a step).
// Every mbarrier wait is bounded; on time-out the CTA records an error code, drains its own copies with a
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
  float lW[N1], lE[N1], lS[N1], lN[N1];
  float qwinv[N1];
};

template <int N1>
constexpr int fused_epb() {
  return (N1 * N1 >= 256) ? 1 : (256 / (N1 * N1));
}

// floats staged per element
template <int N1>
struct Stage {
  static constexpr int NN = N1 * N1;
  static constexpr int Q = 3 * NN, G = 3 * NN, M = 5 * NN, R = 3 * NN, EG = 4 * 5 * N1, NB = 4 * 3 * N1;
  static constexpr int AUXMAX = 5 * NN;
};

template <int N1>
struct SwSmem {
  static constexpr int EPB = fused_epb<N1>();
  static constexpr int NN = N1 * N1;
  struct Buf {
    float q[EPB][3 * NN];
    float G[EPB][3 * NN];
    float met[EPB][5 * NN];
    float aux[EPB][5 * NN];
    float R0[EPB][3 * NN];
    float eg[EPB][4 * 5 * N1];
    float nb[EPB][4][3 * N1];  // neighbour traces (primary-or-secondary side), neighbour node order
  };
  Buf buf[2];
  alignas(8) uint64_t bar[2];
  FConst<N1> C;
  float sT[EPB][4][3][N1];  // own traces
  float sB[EPB][4][3][N1];  // boundary fluxes
  float sF[EPB][3][NN];
  float sG[EPB][3][NN];
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
__global__ void __launch_bounds__(256) sw32_fused(FusedArgs A, FConst<N1> Cg) {
  constexpr int NN = N1 * N1, EPB = fused_epb<N1>();
  // 16-byte granularity of the bulk copies: every staged block is a multiple of 16 bytes for N1 = 4 and 8
  static_assert(N1 == 8, "fused stage: 16-byte bulk-copy granularity and warp-0 lane map are laid out for N1 = 8");
  static_assert(EPB * 4 <= 32, "one warp-0 lane per (element, side) neighbour copy");
  using S = Stage<N1>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SwSmem<N1>& sm = *reinterpret_cast<SwSmem<N1>*>(smem_raw);
  const int tid = threadIdx.x, le = threadIdx.y;
  const int flat = tid + NN * le, nthr = NN * EPB;
  {
    constexpr int NC = sizeof(FConst<N1>) / sizeof(float);
    const float* src = reinterpret_cast<const float*>(&Cg);
    float* dst = reinterpret_cast<float*>(&sm.C);
    for (int t = flat; t < NC; t += nthr) dst[t] = src[t];
  }
  if (flat == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int nchunks = (A.nEl + EPB - 1) / EPB;
  const long long kMaxSpin = 1LL << 20;  // try_wait polls; normal waits end within microseconds

  // warp 0: issue the bulk copies of chunk c into buffer b (lane 0 the element blocks, lanes 4l+s the
  // neighbour traces of element l, side s); the byte count is posted before any copy is issued
  auto issue = [&](int c, int b) {
    const int lane = flat & 31;
    const int e0 = c * EPB;
    const int ne = min(EPB, A.nEl - e0);
    typename SwSmem<N1>::Buf& B = sm.buf[b];
    const int l = lane >> 2, sd = lane & 3;
    ESide es;
    es.nbr = -1;
    if (l < ne && l < EPB) es = A.es[(size_t)(e0 + l) * 4 + sd];
    const bool hasnb = (l < ne && l < EPB) && es.nbr >= 0;
    const unsigned nb = __popc(__ballot_sync(0xffffffffu, hasnb));
    if (lane == 0) {
      uint32_t bytes = (uint32_t)ne * 4u * (S::Q + S::M + A.naux * NN + S::R + S::EG) + nb * 4u * 3u * N1;
      if (A.mode == 2) bytes += (uint32_t)ne * 4u * S::G;
      fence_proxy_async();
      mbar_expect_tx(&sm.bar[b], bytes);
    }
    __syncwarp();
    if (lane == 0) {
      bulk_g2s(&B.q[0][0], A.q + (size_t)e0 * S::Q, ne * 4u * S::Q, &sm.bar[b]);
      if (A.mode == 2) bulk_g2s(&B.G[0][0], A.G + (size_t)e0 * S::G, ne * 4u * S::G, &sm.bar[b]);
      bulk_g2s(&B.met[0][0], A.met + (size_t)e0 * S::M, ne * 4u * S::M, &sm.bar[b]);
      // aux rows are naux*NN per element; the staging rows are 5*NN wide, so copy element by element
      for (int k = 0; k < ne; ++k)
        bulk_g2s(&B.aux[k][0], A.aux + (size_t)(e0 + k) * A.naux * NN, 4u * A.naux * NN, &sm.bar[b]);
      bulk_g2s(&B.R0[0][0], A.R0 + (size_t)e0 * S::R, ne * 4u * S::R, &sm.bar[b]);
      bulk_g2s(&B.eg[0][0], A.eg + (size_t)e0 * S::EG, ne * 4u * S::EG, &sm.bar[b]);
    }
    if (hasnb) {
      fence_proxy_async();
      bulk_g2s(&B.nb[l][sd][0], A.bs_in + (size_t)3 * N1 * (es.nside + 4 * (size_t)es.nbr), 4u * 3u * N1,
               &sm.bar[b]);
    }
  };

  int it = 0;
  int c = blockIdx.x;
  if (c < nchunks && flat < 32) issue(c, 0);
  for (; c < nchunks; c += gridDim.x, ++it) {
    const int b = it & 1;
    const int cn = c + gridDim.x;
    if (cn < nchunks && flat < 32) issue(cn, b ^ 1);  // buffer b^1 was released at the end of iteration it-1
    const bool ok = mbar_wait(&sm.bar[b], (uint32_t)((it >> 1) & 1), kMaxSpin);
    if (__syncthreads_or(!ok)) {
      if (flat == 0) atomicExch(A.err, 1);
      // drain: give outstanding copies of both buffers a second bounded wait, then leave
      mbar_wait(&sm.bar[b], (uint32_t)((it >> 1) & 1), kMaxSpin);
      if (cn < nchunks) mbar_wait(&sm.bar[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1), kMaxSpin);
      return;
    }
    typename SwSmem<N1>::Buf& B = sm.buf[b];
    const int e = c * EPB + le;
    const bool active = e < A.nEl;
    const int i = tid % N1, j = tid / N1;
    // 1. own traces
    if (active) {
      const FConst<N1>& C = sm.C;
      for (int t = tid; t < 4 * 3 * N1; t += NN) {
        const int k = t % N1, v = (t / N1) % 3, side = t / (3 * N1);
        const float* Qv = &B.q[le][v * NN];
        float acc = 0.f;
        if (side == 0 || side == 2) {
          const float* L = (side == 0) ? C.lS : C.lN;
#pragma unroll
          for (int m = 0; m < N1; ++m) acc += L[m] * Qv[k + N1 * m];
        } else {
          const float* L = (side == 1) ? C.lE : C.lW;
#pragma unroll
          for (int m = 0; m < N1; ++m) acc += L[m] * Qv[m + N1 * k];
        }
        sm.sT[le][side][v][k] = acc;
      }
    }
    __syncthreads();
    float qv[3], dxds = 0, dxdp = 0, dyds = 0, dydp = 0, invJ = 0, hn = 0;
    if (active) {
      // 2. fluxes on the 4 sides (threads 0..4*N1-1 of the element)
      if (tid < 4 * N1) {
        const int side = tid / N1, k = tid % N1;
        const ESide es = A.es[(size_t)e * 4 + side];
        const int flags = es.b_flags & 0xff, bb = es.b_flags >> 8;
        const float* egs = &B.eg[le][side * 5 * N1];
        const float nx = egs[k], ny = egs[N1 + k], len = egs[2 * N1 + k], hP = egs[3 * N1 + k], hS = egs[4 * N1 + k];
        float own[3], oth[3], f[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) own[v] = sm.sT[le][side][v][k];
        float sgn = 1.f;
        if (es.nbr >= 0) {
          const int kn = es.a + bb * k;
#pragma unroll
          for (int v = 0; v < 3; ++v) oth[v] = B.nb[le][side][v * N1 + kn];
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
        for (int v = 0; v < 3; ++v) sm.sB[le][side][v][k] = sgn * (f[v] * len);
      }
      // 3. contravariant fluxes
#pragma unroll
      for (int v = 0; v < 3; ++v) qv[v] = B.q[le][v * NN + tid];
      const float* me = &B.met[le][0];
      dxds = me[tid];
      dxdp = me[NN + tid];
      dyds = me[2 * NN + tid];
      dydp = me[3 * NN + tid];
      invJ = me[4 * NN + tid];
      hn = B.aux[le][3 * NN + tid];
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
        sm.sF[le][v][tid] = dydp * xF[v] - dxdp * yF[v];
        sm.sG[le][v][tid] = -dyds * xF[v] + dxds * yF[v];
      }
    }
    __syncthreads();
    if (active) {
      const FConst<N1>& C = sm.C;
      float tend[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        float ds = 0.f, dp = 0.f;
#pragma unroll
        for (int m = 0; m < N1; ++m) ds += C.dS[i + N1 * m] * sm.sF[le][v][m + N1 * j];
        ds += (sm.sB[le][1][v][j] * C.lE[i] + sm.sB[le][3][v][j] * C.lW[i]) * C.qwinv[i];
#pragma unroll
        for (int m = 0; m < N1; ++m) dp += C.dP[j + N1 * m] * sm.sG[le][v][i + N1 * m];
        dp += (sm.sB[le][2][v][i] * C.lN[j] + sm.sB[le][0][v][i] * C.lS[j]) * C.qwinv[j];
        tend[v] = (-ds - dp) * invJ;
      }
      const float* ae = &B.aux[le][0];
      const float dhdx = ae[tid], dhdy = ae[NN + tid], fc = ae[2 * NN + tid];
      float s0 = fc * qv[1] + A.g * qv[2] * dhdx;
      float s1 = -fc * qv[0] + A.g * qv[2] * dhdy;
      float s2 = 0.f;
      if (A.has_drag) {
        s0 -= A.drag * qv[0] / hn;
        s1 -= A.drag * qv[1] / hn;
      }
      if (A.has_relax) {
        const float ts = ae[4 * NN + tid];
        s0 -= qv[0] * ts;
        s1 -= qv[1] * ts;
        s2 -= qv[2] * ts;
      }
      const float* r0 = &B.R0[le][0];
      tend[0] += s0 + r0[tid];
      tend[1] += s1 + r0[NN + tid];
      tend[2] += s2 + r0[2 * NN + tid];
      float* Ge = A.G + (size_t)e * 3 * NN;
      float* qo = A.qout + (size_t)e * 3 * NN;
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const float gg = (A.mode == 2) ? (A.a * B.G[le][v * NN + tid] + tend[v]) : tend[v];
        Ge[v * NN + tid] = gg;
        qv[v] = qv[v] + A.gdt * gg;
        qo[v * NN + tid] = qv[v];
      }
    }
    __syncthreads();  // sF reused for the new state
    if (active) {
#pragma unroll
      for (int v = 0; v < 3; ++v) sm.sF[le][v][tid] = qv[v];
    }
    __syncthreads();
    if (active) {
      const FConst<N1>& C = sm.C;
      for (int t = tid; t < 4 * 3 * N1; t += NN) {
        const int k = t % N1, v = (t / N1) % 3, side = t / (3 * N1);
        const float* Qv = &sm.sF[le][v][0];
        float acc = 0.f;
        if (side == 0 || side == 2) {
          const float* L = (side == 0) ? C.lS : C.lN;
#pragma unroll
          for (int m = 0; m < N1; ++m) acc += L[m] * Qv[k + N1 * m];
        } else {
          const float* L = (side == 1) ? C.lE : C.lW;
#pragma unroll
          for (int m = 0; m < N1; ++m) acc += L[m] * Qv[m + N1 * k];
        }
        A.bs_out[(size_t)3 * N1 * (side + 4 * (size_t)e) + k + N1 * v] = acc;
      }
    }
    __syncthreads();  // buffer b and the scratch arrays are free for the next chunk
  }
}

}  // namespace sw32
}  // namespace selfgpu
