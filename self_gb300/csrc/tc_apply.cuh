// Tensor-core form of the FP32 CGSEM operator apply at N = 7 (pcg_apply_tc): the four derivative-matrix
// contractions of an element tile run as dense GEMMs on the 5th-generation tensor cores (tcgen05.mma kind::tf32,
// operands in shared memory, accumulators in tensor memory) with compensated TF32 products.
//
// A tile is 32 elements = 256 grid lines (one thread per line (e, j): nodes (i, j), i = 0..7).  Each contraction
// is D(M x N) = A(M x K) B(N x K)^T with K = 8 (the contraction index), two MMAs of M = 128 lines:
//   along s (i):  A[(e, j)][k] = u(e, k, j)        -> Du_s(e, i, j) = sum_k D(i, k) u(e, k, j)
//   along p (j):  A[(e, i)][k] = u(e, i, k)        -> Du_p(e, i, j) = sum_k D(j, k) u(e, i, k)
//   then the transposed pair with B(n, k) = D(k, n) on F1 = G11 Du_s + G12 Du_p and F2 = G12 Du_s + G22 Du_p.
// Compensation: A = A_hi + A_lo and D = D_hi + D_lo with every part rounded to TF32 (cvt.rna: 10+1 significant
// bits each, A_hi + A_lo carries 22 bits of A); the B operand holds [D_hi | D_lo] as N = 16 columns, so the two
// MMAs A_hi B and A_lo B give all four products A_x D_y in FP32 accumulators and the epilogue adds the two column
// halves: the products' relative error is about 2^-21 (FP32 is 2^-24), against 2^-11 for one TF32 product.
// Operand layout (no swizzle, K-major): 8-row groups of two 128-byte core matrices (k 0-3, k 4-7); the leading
// byte offset (next core matrix along K) is 144 and the stride byte offset (next 8-row group) 288, padded so that
// the transposed operand writes of a warp (8 rows of 4 groups x 8 columns) fall in 32 distinct banks.  Accumulators:
// TMEM columns 0-63 of a 128-column allocation per CTA (rows 0-127 in columns 0-31, rows 128-255 in columns 32-63;
// s in the first 16 of each, p in the next 16); warp w reads TMEM lanes 32 (w % 4) .. + 31 of column block w / 4.
// Every mbarrier wait is bounded; on time-out (a block-uniform decision) the kernel flags the solve (ioerr
// SELF_ERR_TIMEOUT, done), waits once more for its MMAs, frees its tensor memory and still joins the grid sum.
#pragma once

namespace tc {

constexpr int kTileElems = 32;
constexpr int kTileRows = kTileElems * 8;  // 256 lines = blockDim
constexpr int kLBO = 144, kSBO = 288;         // operand strides (bytes): next core matrix along K, next 8 rows
constexpr int kOpFloats = kTileRows / 8 * kSBO / 4;  // one A operand (256 x 8 TF32, padded)
constexpr int kBFloats = 2 * kSBO / 4;               // one B operand (16 x 8 TF32, padded)
constexpr uint32_t kTmemCols = 128;  // 64 used; the allocation keeps a margin (at most 4 blocks per SM)
constexpr long long kMaxPolls = 1LL << 22;

struct alignas(128) Smem {
  float As_hi[kOpFloats], As_lo[kOpFloats];  // s-direction operand (rows (e, j))
  float Ap_hi[kOpFloats], Ap_lo[kOpFloats];  // p-direction operand (rows (e, i))
  float B1[kBFloats], B2[kBFloats];          // [D_hi | D_lo] for stage 1, [D^T_hi | D^T_lo] for stage 2
  float T[kTileRows * 9];                             // transposes of the p-direction outputs (padded rows)
  uint64_t mbar;
  uint32_t tmem_base;
};

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row r, k) in a K-major operand
__device__ __forceinline__ int opoff(int r, int k) { return (r >> 3) * kSBO + (k >> 2) * kLBO + (r & 7) * 16 + (k & 3) * 4; }

// shared-memory matrix descriptor: start address, LBO, SBO, descriptor version 1 (bits 46-48 = 0b001), base offset
// 0, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// instruction descriptor: FP32 accumulator (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both K-major,
// N = 16 (bits 17-22 = N >> 3), M = 128 (bits 24-28 = M >> 4)
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ float tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void split(float x, float& hi, float& lo) {
  hi = tf32(x);
  lo = tf32(x - hi);
}

__device__ __forceinline__ void mma(uint32_t dtm, uint64_t ad, uint64_t bd, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtm),
      "l"(ad), "l"(bd), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sa(bar))
               : "memory");
}

__device__ __forceinline__ bool wait(uint64_t* bar, uint32_t parity, long long polls) {
  uint32_t done = 0;
  for (long long k = 0; k < polls && !done; ++k)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(sa(bar)), "r"(parity)
        : "memory");
  return done != 0;
}

// 16 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// x (8 values of the thread's line) split into the own-row entries of an s-direction operand (two 16-byte stores
// per part)
__device__ __forceinline__ void put_row(float* hi, float* lo, int r, const float (&x)[8]) {
  float h[8], l[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) split(x[k], h[k], l[k]);
  char* H = reinterpret_cast<char*>(hi);
  char* L = reinterpret_cast<char*>(lo);
  *reinterpret_cast<float4*>(H + opoff(r, 0)) = make_float4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<float4*>(H + opoff(r, 4)) = make_float4(h[4], h[5], h[6], h[7]);
  *reinterpret_cast<float4*>(L + opoff(r, 0)) = make_float4(l[0], l[1], l[2], l[3]);
  *reinterpret_cast<float4*>(L + opoff(r, 4)) = make_float4(l[4], l[5], l[6], l[7]);
}

// x(i) of line (e, j) into rows (e, i), column k = j of a p-direction operand
__device__ __forceinline__ void put_col(float* hi, float* lo, int e, int j, const float (&x)[8]) {
  char* H = reinterpret_cast<char*>(hi);
  char* L = reinterpret_cast<char*>(lo);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    float h, l;
    split(x[i], h, l);
    *reinterpret_cast<float*>(H + opoff(e * 8 + i, j)) = h;
    *reinterpret_cast<float*>(L + opoff(e * 8 + i, j)) = l;
  }
}

}  // namespace tc

template <int NF>
__global__ void __launch_bounds__(tc::kTileRows) pcg_apply_tc(const float* __restrict__ w, const float* __restrict__ vold,
                                                              float* __restrict__ vnew, const int* __restrict__ src,
                                                              const float* __restrict__ fac, float* __restrict__ z,
                                                              int nEl, CGConst<8, float> Cg, CGScalars* S,
                                                              double* __restrict__ partial,
                                                              unsigned int* __restrict__ ticket) {
  static_assert(tc::kTileRows == kRedThreads, "one thread per line, 256 threads: the grid sums assume it");
  if (S->done) return;
  constexpr int NN = 64;
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  tc::Smem& sm = *reinterpret_cast<tc::Smem*>(tc_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  // B operands: stage 1 rows n: D(n, k) (n < 8: TF32 part, n >= 8: remainder); stage 2: D(k, n)
  for (int q = tid; q < 128; q += kRedThreads) {
    const int n = q >> 3, k = q & 7, nn = n & 7;
    float h1, l1, h2, l2;
    tc::split(Cg.D[nn + 8 * k], h1, l1);  // D(nn, k), column-major
    tc::split(Cg.D[k + 8 * nn], h2, l2);  // D(k, nn)
    *reinterpret_cast<float*>(reinterpret_cast<char*>(sm.B1) + tc::opoff(n, k)) = n < 8 ? h1 : l1;
    *reinterpret_cast<float*>(reinterpret_cast<char*>(sm.B2) + tc::opoff(n, k)) = n < 8 ? h2 : l2;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::sa(&sm.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::sa(&sm.tmem_base)),
                 "r"(tc::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = sm.tmem_base;
  const int r = tid;                    // this thread's line: element le, row j
  const int le = r >> 3, j = r & 7;
  // TMEM address of this warp's lanes and column block: lane field 32 (warp % 4), columns 32 * (warp / 4)
  const uint32_t tw = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * (warp >> 2));
  const uint64_t dB1 = tc::sdesc(tc::sa(sm.B1)), dB2 = tc::sdesc(tc::sa(sm.B2));
  const bool first = S->iter == 0;
  const float beta = first ? 0.f : S->beta32;
  const int ngroups = (nEl + tc::kTileElems - 1) / tc::kTileElems;
  uint32_t phase = 0;
  bool failed = false;
  float pa = 0.f;
  auto issue = [&](uint64_t dB) {  // one thread: s and p MMAs of both halves (hi then lo with accumulation)
    tc::fence_after();
    for (int h = 0; h < 2; ++h) {
      const uint32_t off = (uint32_t)(h * 128 / 8 * tc::kSBO);  // 16 row groups per half
      const uint32_t dcol = tmem + (uint32_t)(32 * h);
      tc::mma(dcol, tc::sdesc(tc::sa(sm.As_hi) + off), dB, 0);
      tc::mma(dcol, tc::sdesc(tc::sa(sm.As_lo) + off), dB, 1);
      tc::mma(dcol + 16, tc::sdesc(tc::sa(sm.Ap_hi) + off), dB, 0);
      tc::mma(dcol + 16, tc::sdesc(tc::sa(sm.Ap_lo) + off), dB, 1);
    }
    tc::commit(&sm.mbar);
  };
  // reads this thread's s row (own line) and p row (a column line, transposed through T into the own line)
  auto gather = [&](float (&s_out)[8], float (&p_out)[8]) {
    float a[16], b[16];
    tc::ld16(tw, a);
    tc::ld16(tw + 16, b);
    tc::ld_wait();
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      s_out[k] = a[k] + a[k + 8];
      sm.T[(le * 8 + k) * 9 + j] = b[k] + b[k + 8];  // row (le, i = j) holds column line values at j' = k
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 8; ++k) p_out[k] = sm.T[(le * 8 + j) * 9 + k];
  };
  for (int g = blockIdx.x; g < ngroups && !failed; g += gridDim.x) {
    const int e = g * tc::kTileElems + le;
    const bool active = e < nEl;
    const size_t l0 = (size_t)e * NN + (size_t)8 * j;
    float u[8];
    if (active) {
      const float* fe = fac + (size_t)e * NF * NN + (size_t)8 * j;
#pragma unroll
      for (int f = 0; f < 4; ++f) prefetch_l2(fe + f * NN);
      int sl[8];
      float wl[8], vl[8], vn[8];
      load_line<8>(src + l0, sl);
      load_line<8>(w + l0, wl);
      if (first) {
#pragma unroll
        for (int i = 0; i < 8; ++i) vl[i] = 0.f;
      } else {
        load_line<8>(vold + l0, vl);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        vn[i] = first ? wl[i] : wl[i] + beta * vl[i];
        u[i] = sl[i] == (int)(l0 + i) ? vn[i] : (first ? w[sl[i]] : w[sl[i]] + beta * vold[sl[i]]);
      }
      store_line<8>(vnew + l0, vn);
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) u[i] = 0.f;
    }
    // stage 1 operands: u along s (own row) and along p (column k = j of rows (le, i))
    tc::put_row(sm.As_hi, sm.As_lo, r, u);
    tc::put_col(sm.Ap_hi, sm.Ap_lo, le, j, u);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) issue(dB1);
    if (__syncthreads_or(!tc::wait(&sm.mbar, phase, tc::kMaxPolls))) {  // block-uniform decision
      failed = true;
      break;
    }
    phase ^= 1u;
    tc::fence_after();
    float us[8], up[8];
    gather(us, up);
    // fluxes and stage 2 operands (the stage-1 MMAs have read their operands: the commit arrived)
    float F1[8], F2[8];
    if (active) {
      const float* fe = fac + (size_t)e * NF * NN + (size_t)8 * j;
      float G11[8], G12[8], G22[8];
      load_line<8>(fe, G11);
      load_line<8>(fe + NN, G12);
      load_line<8>(fe + 2 * NN, G22);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        F1[i] = G11[i] * us[i] + G12[i] * up[i];
        F2[i] = G12[i] * us[i] + G22[i] * up[i];
      }
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) F1[i] = F2[i] = 0.f;
    }
    tc::put_row(sm.As_hi, sm.As_lo, r, F1);
    tc::put_col(sm.Ap_hi, sm.Ap_lo, le, j, F2);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();  // also: every thread's stage-1 TMEM reads and T reads are done
    if (tid == 0) issue(dB2);
    if (__syncthreads_or(!tc::wait(&sm.mbar, phase, tc::kMaxPolls))) {
      failed = true;
      break;
    }
    phase ^= 1u;
    tc::fence_after();
    float a1[8], a2[8];
    gather(a1, a2);  // (D^T F1)(i, j) on the own line, (D^T F2)(i, j) transposed into it
    if (active) {
      const float* fe = fac + (size_t)e * NF * NN + (size_t)8 * j;
      float Mv[8], Lu[8];
      load_line<8>(fe + 3 * NN, Mv);
#pragma unroll
      for (int i = 0; i < 8; ++i) Lu[i] = -(a1[i] + a2[i]) - Mv[i] * u[i];
      if (NF == 6) {
        float B1[8], B2[8];
        load_line<8>(fe + 4 * NN, B1);
        load_line<8>(fe + 5 * NN, B2);
#pragma unroll
        for (int i = 0; i < 8; ++i) Lu[i] -= B1[i] * us[i] + B2[i] * up[i];
      }
      store_line<8>(z + l0, Lu);
#pragma unroll
      for (int i = 0; i < 8; ++i) pa += u[i] * Lu[i];
    }
    tc::fence_before();
    __syncthreads();  // T, the operands and TMEM are reused by the next tile
  }
  if (failed) {  // flag the solve, let the MMAs in flight finish, free the tensor memory
    if (tid == 0) {
      S->ioerr = SELF_ERR_TIMEOUT;
      S->done = 1;
    }
    tc::wait(&sm.mbar, phase, tc::kMaxPolls);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kTmemCols) : "memory");
  }
  // a failed block still joins the grid sum, so the ticket protocol completes (the solve is flagged done)
  const float acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, float>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->vz = tot[0];
    S->alpha = S->num / tot[0];
    S->alpha32 = (float)S->alpha;
  }
}
