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
// fused PCG.  The N^2 sub-quads of one element are applied together from shared memory:
//   corner (a, b) of sub-quad (si, pj):  us = (u(si+1, pj+b) - u(si, pj+b)) / 2,  up = (u(si+a, pj+1) - u(si+a, pj)) / 2
//     F1 = G11 us + G12 up,  F2 = G12 us + G22 up  (G = folded metric factors of the bilinear sub-quad, k = 1)
//   node (i, j) sums, over the sub-quads (i-1, j-1), (i, j-1), (i-1, j), (i, j) that contain it (the reference's
//   linear element order), -( +-(F1(0, b) + F1(1, b)) / 2 + +-(F2(a, 0) + F2(a, 1)) / 2 )
// which is FluxDivergence_CGsemPreconditioner_2D (:480-555) with the N = 1 Gauss-Lobatto derivative matrix
// (entries -1/2, 1/2) and weights (1, 1).
// One inner CG iteration is three launches (q1_apply_fused, cg_dss_mask with the linear groups, pcl_update);
// pcl_start maps the outer residual in and pc_num forms w, <r, w> and the outer beta from the inner solution.
// Dirichlet lift: the reference's inner CG keeps the mapped residual's values on the linear mesh's Dirichlet nodes
// (w = r, v = w + c v, and MatrixAction's UnMask skips Dirichlet nodes), so every matrix action sees those values
// there.  They are zero when the spectral residual is (its own Dirichlet nodes); where the linear mesh has Dirichlet
// nodes the spectral mesh does not (a Neumann boundary, nodes its position search left split) rd holds them and
// the operator adds them to the gathered direction, outside the masked <v, Lv>.

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
  constexpr int NQ = 4 * N * N;  // sub-quad corners per element
  constexpr int EPB = cg_epb<N1>();
  static_assert(EPB * NN <= kRedThreads, "one element group per block pass");
  __shared__ R su[EPB][NN];
  __shared__ R sF1[EPB][NQ];
  __shared__ R sF2[EPB][NQ];
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
    R u = 0, ud = 0;
    if (active) {
      const int sl = src[l];
      const R ws = w[sl];
      u = first ? ws : ws + beta * vold[sl];
      vnew[l] = first ? w[l] : w[l] + beta * vold[l];
      if (rd) ud = rd[l];
      su[le][tid] = u + ud;
    }
    __syncthreads();
    // sub-quad corners: fluxes F1, F2
    for (int c = threadIdx.x; c < EPB * NQ; c += kRedThreads) {
      const int ee = c / NQ, cc = c - ee * NQ;
      const int e2 = g * EPB + ee;
      if (e2 >= nEl) continue;
      const int q = cc >> 2, a = cc & 1, b = (cc >> 1) & 1;
      const int si = q % N, pj = q / N;
      const R* U = su[ee];
      const R us = R(0.5) * (U[(si + 1) + N1 * (pj + b)] - U[si + N1 * (pj + b)]);
      const R up = R(0.5) * (U[(si + a) + N1 * (pj + 1)] - U[(si + a) + N1 * pj]);
      const R* fe = fac + (size_t)e2 * 3 * NQ;
      const R G11 = fe[cc], G12 = fe[NQ + cc], G22 = fe[2 * NQ + cc];
      sF1[ee][cc] = G11 * us + G12 * up;
      sF2[ee][cc] = G12 * us + G22 * up;
    }
    __syncthreads();
    if (active) {
      R Lu = 0;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int si = i - 1 + (t & 1), pj = j - 1 + (t >> 1);
        if (si < 0 || si >= N || pj < 0 || pj >= N) continue;
        const int a = i - si, b = j - pj;
        const R* F1 = &sF1[le][4 * (si + N * pj)];
        const R* F2 = &sF2[le][4 * (si + N * pj)];
        const R d1 = (a ? R(0.5) : R(-0.5)) * (F1[2 * b] + F1[1 + 2 * b]);
        const R d2 = (b ? R(0.5) : R(-0.5)) * (F2[a] + F2[a + 2]);
        Lu += -(d1 + d2);
      }
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
