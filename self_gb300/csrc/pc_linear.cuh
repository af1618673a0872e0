// Linear-FEM preconditioner of the CGSEM 2-D PCG (CGsemPreconditioner_2D_Class.f90, built on the mesh of
// QuadMeshClass.f90 ConstructLinearMeshFromOther :1863-2092), device kernels.  Included by cg2d.cu inside
// namespace selfgpu::cg after the fused PCG kernels.
//
// The reference's preconditioner mesh has one bilinear element per GLL sub-quad of every spectral element
// (nEl*N^2 elements, corner nodes = the GLL nodes).  Here it stays in the spectral element's own L-vector layout:
// a vector of the linear mesh is an L-vector of the original mesh (a GLL node of one spectral element stands for
// its 1-4 sub-quad copies, which always share one position), with the linear mesh's own primary-copy gather
// (UnMask), direct-stiffness groups (GlobalSum + Mask) and Dirichlet set, compiled on the host from the
// reference's position-based node identification; the inner CG uses the element-local <v, Lv> trick of the
// fused PCG.
// Operator: FluxDivergence_CGsemPreconditioner_2D (:480-555) on one bilinear sub-quad, with the N = 1
// Gauss-Lobatto derivative matrix (entries -1/2, 1/2) and weights (1, 1), is a symmetric 4 x 4 matrix; summed over
// the sub-quads of a spectral element it is a symmetric 9-point stencil on the element's GLL grid.  The host
// assembles it once (k = 1, the preconditioner's fluxCoeff) and stores, per node, the coefficients of itself and
// of its E, N, NE and NW neighbours; the W, S, SW and SE coefficients are those of the neighbour in the opposite
// direction (symmetry).  Per node this is 9 multiply-adds: the FP64 pipe, far narrower than the FP32 one on this
// part, bounds the FP64 form, so the fluxes are not recomputed at every sub-quad corner.
// One inner CG iteration is three launches (q1_apply_fused, cg_dss_mask_pairs with the linear groups, pcl_update);
// pcl_start maps the outer residual in and pc_num forms w, <r, w> and the outer beta from the inner solution.
// Dirichlet lift: the reference's inner CG keeps the mapped residual's values on the linear mesh's Dirichlet nodes
// (w = r, v = w + c v, and MatrixAction's UnMask skips Dirichlet nodes), so every matrix action sees those values
// there.  They are zero when the spectral residual is (its own Dirichlet nodes); where the linear mesh has Dirichlet
// nodes the spectral mesh does not (a Neumann boundary, nodes its position search left split) rd holds them and
// the operator adds them to the gathered direction, outside the masked <v, Lv>.

// stencil coefficient slots per node
constexpr int kQ1Self = 0, kQ1E = 1, kQ1N = 2, kQ1NE = 3, kQ1NW = 4, kQ1Slots = 5;

template <int N1, typename R>
__global__ void __launch_bounds__(kRedThreads) q1_apply_fused(const R* __restrict__ w, const R* __restrict__ vold,
                                                              R* __restrict__ vnew, const int* __restrict__ src,
                                                              const R* __restrict__ rd, const R* __restrict__ fac,
                                                              R* __restrict__ z, int nEl,
                                                              const CGScalars* __restrict__ S, CGScalars* SL,
                                                              double* __restrict__ partial,
                                                              unsigned int* __restrict__ ticket) {
  if (S->done || SL->done) return;
  constexpr int N = N1 - 1;
  constexpr int NN = N1 * N1;
  constexpr int EPB = cg_epb<N1>();
  static_assert(EPB * NN <= kRedThreads, "one element group per block pass");
  __shared__ R su[EPB][NN];
  __shared__ R sc[EPB][kQ1Slots - 1][NN];  // E, N, NE, NW coefficients (read by the neighbours)
  const int tid = threadIdx.x % NN, le = threadIdx.x / NN;
  const bool first = SL->iter == 0;
  const R beta = first ? R(0) : (sizeof(R) == 4 ? (R)SL->beta32 : (R)SL->beta);
  const int i = tid % N1, j = tid / N1;
  const int ngroups = (nEl + EPB - 1) / EPB;
  R pa = 0;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int e = g * EPB + le;
    const bool active = le < EPB && e < nEl;
    const size_t l = (size_t)e * NN + tid;
    R u = 0, c0 = 0, cE = 0, cN = 0, cNE = 0, cNW = 0;
    if (active) {
      const R* fe = fac + (size_t)e * kQ1Slots * NN;
      c0 = fe[kQ1Self * NN + tid];
      cE = fe[kQ1E * NN + tid];
      cN = fe[kQ1N * NN + tid];
      cNE = fe[kQ1NE * NN + tid];
      cNW = fe[kQ1NW * NN + tid];
      const int sl = src[l];
      const R wl = w[l];
      const R vn = first ? wl : wl + beta * vold[l];
      vnew[l] = vn;
      u = sl == (int)l ? vn : (first ? w[sl] : w[sl] + beta * vold[sl]);
      su[le][tid] = rd ? u + rd[l] : u;
      sc[le][kQ1E - 1][tid] = cE;
      sc[le][kQ1N - 1][tid] = cN;
      sc[le][kQ1NE - 1][tid] = cNE;
      sc[le][kQ1NW - 1][tid] = cNW;
    }
    __syncthreads();
    if (active) {
      const R* U = su[le];
      R Lu = c0 * U[tid];
      if (i < N) Lu += cE * U[tid + 1];
      if (j < N) Lu += cN * U[tid + N1];
      if (i < N && j < N) Lu += cNE * U[tid + N1 + 1];
      if (i > 0 && j < N) Lu += cNW * U[tid + N1 - 1];
      if (i > 0) Lu += sc[le][kQ1E - 1][tid - 1] * U[tid - 1];
      if (j > 0) Lu += sc[le][kQ1N - 1][tid - N1] * U[tid - N1];
      if (i > 0 && j > 0) Lu += sc[le][kQ1NE - 1][tid - N1 - 1] * U[tid - N1 - 1];
      if (i < N && j > 0) Lu += sc[le][kQ1NW - 1][tid - N1 + 1] * U[tid - N1 + 1];
      z[l] = Lu;
      pa += u * Lu;
    }
    __syncthreads();  // the next group reuses the scratch arrays
  }
  const R acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, R>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    SL->vz = tot[0];
    SL->alpha = SL->num / tot[0];
    SL->alpha32 = (float)SL->alpha;
  }
}

// r_l = MapFromOrigToPC(UnMask(r)) in masked form: every primary copy of a non-Dirichlet node of the linear mesh
// takes the spectral residual's value there (r[src[k]], the spectral primary copy), every other copy 0; u_l = 0;
// the inner CG's r0 and num = <r_l, r_l>; a fresh inner solve (iter 0); with rd, the Dirichlet lift (the
// residual's values on the copies dlift marks).
template <typename R>
__global__ void __launch_bounds__(kRedThreads) pcl_start(const R* __restrict__ r, const int* __restrict__ src,
                                                         const unsigned char* __restrict__ lprim,
                                                         const unsigned char* __restrict__ dlift, R* __restrict__ rl,
                                                         R* __restrict__ ul, R* __restrict__ rd, size_t n,
                                                         const CGScalars* __restrict__ S, CGScalars* SL,
                                                         double* __restrict__ partial, unsigned int* __restrict__ ticket) {
  if (S->done) return;
  R pa = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const R rk = lprim[k] ? r[src[k]] : R(0);
    rl[k] = rk;
    ul[k] = R(0);
    if (rd) rd[k] = dlift[k] ? r[src[k]] : R(0);
    pa += rk * rk;
  }
  const R acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, R>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    SL->num = tot[0];
    SL->rr = sqrt(tot[0]);
    SL->r0 = SL->rr;
    SL->iter = 0;
    SL->done = (SL->maxIters <= 0 || tot[0] == 0.0) ? 1 : 0;
  }
}

// u_l += a v_l, r_l -= a z_l, num = <r_l, r_l> (the reference's w = r), stop at ||r_l|| / r0 < TOL or maxIters
template <typename R>
__global__ void __launch_bounds__(kRedThreads) pcl_update(R* __restrict__ ul, R* __restrict__ rl,
                                                          const R* __restrict__ vl, const R* __restrict__ zl, size_t n,
                                                          const CGScalars* __restrict__ S, CGScalars* SL,
                                                          double* __restrict__ partial, unsigned int* __restrict__ ticket) {
  if (S->done || SL->done) return;
  const R a = sizeof(R) == 4 ? (R)SL->alpha32 : (R)SL->alpha;
  R prr = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    ul[k] += a * vl[k];
    const R rk = rl[k] - a * zl[k];
    rl[k] = rk;
    prr += rk * rk;
  }
  const R acc[1] = {prr};
  double tot[1];
  if (!grid_sums_last<1, R>(acc, partial, ticket, tot) || threadIdx.x != 0) return;
  SL->den = SL->num;
  SL->num = tot[0];
  SL->beta = SL->num / SL->den;
  SL->beta32 = (float)SL->beta;
  SL->iter += 1;
  SL->rr = sqrt(tot[0]);
  if (SL->rr / SL->r0 < SL->tol || SL->iter >= SL->maxIters) SL->done = 1;
}

// pcl_update over 16-byte groups of consecutive nodes (float4 / double2; the L-vector length is a multiple of the
// group when (N+1)^2 nEl is): each thread keeps two groups of its 4 streams in flight
template <typename R, typename V>
__global__ void __launch_bounds__(kRedThreads) pcl_update_vec(V* __restrict__ ul, V* __restrict__ rl,
                                                              const V* __restrict__ vl, const V* __restrict__ zl,
                                                              size_t nv, const CGScalars* __restrict__ S, CGScalars* SL,
                                                              double* __restrict__ partial,
                                                              unsigned int* __restrict__ ticket) {
  static_assert(sizeof(V) == 16 && sizeof(V) % sizeof(R) == 0, "16-byte groups");
  constexpr int L = sizeof(V) / sizeof(R);
  if (S->done || SL->done) return;
  const R a = sizeof(R) == 4 ? (R)SL->alpha32 : (R)SL->alpha;
  R prr = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  constexpr int U = 2;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += U * stride) {
    V uu[U], vv[U], rr[U], zz[U];
    bool ok[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const size_t x = k + q * stride;
      ok[q] = x < nv;
      if (!ok[q]) continue;
      uu[q] = ul[x];
      vv[q] = vl[x];
      rr[q] = rl[x];
      zz[q] = zl[x];
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      if (!ok[q]) continue;
      R us[L], vs[L], rs[L], zs[L];
      memcpy(us, &uu[q], 16);
      memcpy(vs, &vv[q], 16);
      memcpy(rs, &rr[q], 16);
      memcpy(zs, &zz[q], 16);
#pragma unroll
      for (int c = 0; c < L; ++c) {
        us[c] += a * vs[c];
        rs[c] = rs[c] - a * zs[c];
        prr += rs[c] * rs[c];
      }
      V t;
      memcpy(&t, us, 16);
      ul[k + q * stride] = t;
      memcpy(&t, rs, 16);
      rl[k + q * stride] = t;
    }
  }
  const R acc[1] = {prr};
  double tot[1];
  if (!grid_sums_last<1, R>(acc, partial, ticket, tot) || threadIdx.x != 0) return;
  SL->den = SL->num;
  SL->num = tot[0];
  SL->beta = SL->num / SL->den;
  SL->beta32 = (float)SL->beta;
  SL->iter += 1;
  SL->rr = sqrt(tot[0]);
  if (SL->rr / SL->r0 < SL->tol || SL->iter >= SL->maxIters) SL->done = 1;
}

// w = MapFromPCToOrig(UnMask(u_l)) in the spectral mesh's masked form: each spectral primary copy (src[k] == k)
// takes u_l at its linear primary copy (lsrc[k]), the other copies 0; num = <r, w>, and the outer beta = num / den
// after the first outer iteration.
template <typename R>
__global__ void __launch_bounds__(kRedThreads) pc_num(const R* __restrict__ r, const R* __restrict__ ul,
                                                      const int* __restrict__ src, const int* __restrict__ lsrc,
                                                      R* __restrict__ w, size_t n, CGScalars* S,
                                                      double* __restrict__ partial, unsigned int* __restrict__ ticket) {
  if (S->done) return;
  R pa = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const R wk = src[k] == (int)k ? ul[lsrc[k]] : R(0);
    w[k] = wk;
    pa += r[k] * wk;
  }
  const R acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, R>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->num = tot[0];
    if (S->iter > 0) {
      S->beta = S->num / S->den;
      S->beta32 = (float)S->beta;
    }
  }
}
