// FP32 inner PCG on the compact node layout: one value per unknown instead of one per element-local copy.
//
// The masked L-vectors of the element-local form store every shared node once per element (zeros at the
// non-primary copies) and need a separate direct-stiffness pass (cg_dss_mask_pairs) of scattered 4-byte accesses.
// Here the Krylov vectors hold the unknowns only, grouped by mesh entity:
//   [ element interiors: nEl x M^2, by pass groups of the apply (interior_index)          ]  nInt
//   [ two-sided edges:   M nodes each, in the primary element's order along its side     ]  nE2 M
//   [ one-sided edges (boundary sides without a Dirichlet condition)                     ]  nE1 M
//   [ corners (mesh vertices without a Dirichlet condition)                              ]  nC
//   [ padding to a multiple of 4 (zero, never updated)                                   ]
// with M = N1 - 2 nodes inside an edge.  Dirichlet nodes are not unknowns and do not appear.  Each element carries
// a 48-byte descriptor (3 int4): its four sides' edge codes (id << 2 | slot << 1 | flip, -1 for a Dirichlet side),
// its four corners' codes (id << 1 | owner, -1 for a Dirichlet corner) and its four corners' contribution slots.
// The element factors are stored line-interleaved (factor_index) so that a warp's loads are contiguous; on affine
// meshes one value per node (k w_i w_j) and four per element replace the four factors per node.
//
// Two kernels per iteration.  pcg_apply_compact_f32 (one thread per grid line, warp-synchronous when a warp holds
// whole elements; D from the constant bank): v_new = w + beta v_old, the element operator, and its output written
// without any summation: interior rows straight into the z vector's interior block, an edge side's M values into
// its slot (primary side 0, secondary side 1) of the edge contribution block, a corner's value into its slot of the
// corner block (slots in the order of the corner's copies in the shared-node group, primary first).
// pcg_update_compact forms the assembled z node by node (interior = the value, two-sided edge = slot 0 + slot 1,
// one-sided edge = slot 0, corner = 0 + slots in order: the direct-stiffness sums of cg_dss_mask_pairs in the same
// summation order) and updates u, r, w with the grid sums of <r, w> and <r, r>.
// Included by cg2d.cu inside namespace selfgpu::cg, after the reductions, CGScalars and the line helpers.
#pragma once

struct CompactView {
  const int4* __restrict__ desc;  // 3 per element: edge codes (S, E, N, W), corner codes, corner slots (SW, SE, NE, NW)
  const int* __restrict__ coff;   // corner c's slots: [coff[c], coff[c + 1])
  int nInt, nE2, nE1, nC, ngp;    // block sizes (nodes; edges; corners) and the padded vector length
  int nEl;
};

// Values a thread moves at once along a line: 4 (16 bytes), 2 or 1, whichever divides the line.
template <int K>
constexpr int chunk_of() {
  return K % 4 == 0 ? 4 : (K % 2 == 0 ? 2 : 1);
}

// Interior node (ii, jj) (0-based inside the element, ii along s) of element e in the interior block.  The block is
// laid out by pass groups of EPL elements (the elements one block pass of the apply covers) so that the threads of
// a warp, one per grid line jj of consecutive elements, read a chunk of consecutive interior values each from one
// contiguous stretch: inside group g (ne elements) chunk c = ii / CH, then element, then jj, then ii % CH.
template <int N1>
__host__ __device__ __forceinline__ int interior_index(int e, int ii, int jj, int nEl) {
  constexpr int M = N1 - 2, EPL = line_epb<N1>(), CH = chunk_of<M>();
  const int g = e / EPL, le = e - g * EPL, ne = (nEl - g * EPL < EPL) ? nEl - g * EPL : EPL;
  const int c = ii / CH, r = ii - c * CH;
  return g * EPL * M * M + ((c * ne + le) * M + jj) * CH + r;
}

// The FP32 element factors, line-interleaved for the compact apply: factor f at node (i, line t) of element
// e = g EPL + le (line = le N1 + t) sits at chunk c = i / CH of the line, the lines of a pass group consecutive, so a
// warp's chunk loads are contiguous.  The last group is padded to EPL elements.
template <int N1>
__host__ __device__ __forceinline__ size_t factor_index(int NF, int g, int f, int i, int line) {
  constexpr int LPG = line_epb<N1>() * N1, CH = chunk_of<N1>();
  const int c = i / CH, r = i - c * CH;
  return ((((size_t)g * NF + f) * (N1 / CH) + c) * LPG + line) * CH + r;
}

template <int CH>
__device__ __forceinline__ void ld_chunk(const float* __restrict__ p, float* x) {
  if constexpr (CH == 4) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
  } else if constexpr (CH == 2) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    x[0] = v.x, x[1] = v.y;
  } else {
    x[0] = p[0];
  }
}

template <int CH>
__device__ __forceinline__ void ld_chunk(const double* __restrict__ p, double* x) {
#pragma unroll
  for (int c = 0; c + 1 < CH; c += 2) {
    const double2 v = *reinterpret_cast<const double2*>(p + c);
    x[c] = v.x, x[c + 1] = v.y;
  }
  if constexpr (CH == 1) x[0] = p[0];
}

template <int CH>
__device__ __forceinline__ void st_chunk(double* __restrict__ p, const double* x) {
#pragma unroll
  for (int c = 0; c + 1 < CH; c += 2) *reinterpret_cast<double2*>(p + c) = make_double2(x[c], x[c + 1]);
  if constexpr (CH == 1) p[0] = x[0];
}

template <int CH>
__device__ __forceinline__ void st_chunk(float* __restrict__ p, const float* x) {
  if constexpr (CH == 4)
    *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
  else if constexpr (CH == 2)
    *reinterpret_cast<float2*>(p) = make_float2(x[0], x[1]);
  else
    p[0] = x[0];
}

// Compact indices of the N1 nodes (i, t), i = 0..N1-1, of line t of element e: gi = the unknown (-1: Dirichlet),
// zi = where the element's operator value goes in the contribution space (interiors | edge slots | corner slots),
// bit i of own set when this element writes the node's new direction value (the unknown's primary copy).
// d0, d1, d2 = the element's descriptor.
template <int N1>
__device__ __forceinline__ void compact_line(const CompactView& V, int e, int t, int4 d0, int4 d1, int4 d2,
                                             int (&gi)[N1], int (&zi)[N1], unsigned& own) {
  constexpr int M = N1 - 2;
  const int nEM = (V.nE2 + V.nE1) * M;
  own = 0u;
  auto edge = [&](int code, int k, int q) {
    if (code < 0) {
      gi[q] = -1;
      zi[q] = -1;
      return;
    }
    const int id = code >> 2, slot = (code >> 1) & 1, kc = (code & 1) ? M - 1 - k : k;
    gi[q] = V.nInt + id * M + kc;
    zi[q] = V.nInt + (2 * id + slot) * M + kc;
    if (slot == 0) own |= 1u << q;
  };
  auto corner = [&](int code, int fs, int q) {
    if (code < 0) {
      gi[q] = -1;
      zi[q] = -1;
      return;
    }
    gi[q] = V.nInt + nEM + (code >> 1);
    zi[q] = V.nInt + 2 * nEM + fs;
    if (code & 1) own |= 1u << q;
  };
  if (t == 0 || t == N1 - 1) {  // south (j = 0) or north (j = N) side: corners at i = 0, N
    const bool s = t == 0;
    corner(s ? d1.x : d1.w, s ? d2.x : d2.w, 0);
    corner(s ? d1.y : d1.z, s ? d2.y : d2.z, N1 - 1);
#pragma unroll
    for (int i = 1; i <= M; ++i) edge(s ? d0.x : d0.z, i - 1, i);
  } else {  // west (i = 0) and east (i = N) side nodes, interior row t - 1 between them
    edge(d0.w, t - 1, 0);
    edge(d0.y, t - 1, N1 - 1);
#pragma unroll
    for (int i = 1; i <= M; ++i) {
      gi[i] = interior_index<N1>(e, i - 1, t - 1, V.nEl);
      zi[i] = gi[i];
      own |= 1u << i;
    }
  }
}

// v_new = w + beta v_old on the compact layout, z = L(v_new) per element into the contribution space, partial sums
// of <v_new, z>: the line operator of pcg_apply_fused_f32 with compact gathers and slot stores.
// Affine elements: factor f < 3 of node (i, j) = kw(i, j) ec[e].f, the mass factor = ec[e].w w_i w_j (see
// build_factors); one streamed value per node.
template <int N1>
struct AffineOp {
  const float* __restrict__ kwT;  // k w_i w_j, line-interleaved as factor_index with one factor
  const float4* __restrict__ ec;  // (c11, c12, c22, lambda J) per element
  float ww[N1 * N1];              // w_i w_j, node i + N1 j
};

template <int N1, int NF, bool AFF>
__global__ void __launch_bounds__(kRedThreads) pcg_apply_compact_f32(const float* __restrict__ w,
                                                                     const float* __restrict__ vold,
                                                                     float* __restrict__ vnew, CompactView V,
                                                                     const float* __restrict__ facT,
                                                                     AffineOp<N1> A, float* __restrict__ zc,
                                                                     CGConst<N1, float> Cg, CGScalars* S,
                                                                     double* __restrict__ partial,
                                                                     unsigned int* __restrict__ ticket) {
  static_assert(!AFF || NF == 4, "affine factors: Helmholtz operator");
  if (S->done) return;
  constexpr int M = N1 - 2;
  constexpr int EPL = line_epb<N1>();
  constexpr int LS = N1 + 1;
  constexpr int CF = chunk_of<N1>(), CI = chunk_of<M>();
  __shared__ float X[EPL * N1 * LS];
  __shared__ float Y[EPL * N1 * LS];
  __shared__ float WW[AFF ? N1 * N1 : 1];
  if constexpr (AFF)
    for (int k = threadIdx.x; k < N1 * N1; k += blockDim.x) WW[k] = A.ww[k];
  __syncthreads();
  const int nEl = V.nEl;
  const int le = threadIdx.x / N1, t = threadIdx.x - le * N1;
  const int line = le * N1 + t;
  const bool first = S->iter == 0;
  const float beta = first ? 0.f : S->beta32;
  const int ngroups = (nEl + EPL - 1) / EPL;
  const bool irow = t > 0 && t < N1 - 1;  // the line crosses the interior (row t - 1 of the interior block)
  float pa = 0.f;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int e = g * EPL + le;
    const bool active = le < EPL && e < nEl;
    auto fl = [&](int f, float (&G)[N1]) {
      if constexpr (AFF) {
        const float4 c4 = A.ec[e];
        if (f == 3) {
#pragma unroll
          for (int i = 0; i < N1; ++i) G[i] = c4.w * WW[i + N1 * t];
        } else {
          const float cf = f == 0 ? c4.x : (f == 1 ? c4.y : c4.z);
#pragma unroll
          for (int c = 0; c < N1 / CF; ++c) ld_chunk<CF>(A.kwT + factor_index<N1>(1, g, 0, c * CF, line), G + c * CF);
#pragma unroll
          for (int i = 0; i < N1; ++i) G[i] *= cf;
        }
      } else {
#pragma unroll
        for (int c = 0; c < N1 / CF; ++c) ld_chunk<CF>(facT + factor_index<N1>(NF, g, f, c * CF, line), G + c * CF);
      }
    };
    float u[N1], Lu[N1];
    int ib = 0, cstride = 0;  // the interior row's first chunk and the distance between its chunks
    if (active) {
#pragma unroll
      for (int f = 0; f < (AFF ? 1 : 4); ++f)  // read two barriers later
#pragma unroll
        for (int c = 0; c < N1 / CF; ++c)
          prefetch_l2(AFF ? A.kwT + factor_index<N1>(1, g, 0, c * CF, line)
                          : facT + factor_index<N1>(NF, g, f, c * CF, line));
      int gi[N1], zi[N1];
      unsigned own;
      compact_line<N1>(V, e, t, V.desc[3 * e], V.desc[3 * e + 1], V.desc[3 * e + 2], gi, zi, own);
      float wl[N1], vl[N1];
      if (irow) {  // interior values in chunks, the two side nodes gathered
        const int ne = min(EPL, nEl - g * EPL);
        ib = interior_index<N1>(e, 0, t - 1, nEl);
        cstride = ne * M * CI;
#pragma unroll
        for (int c = 0; c < M / CI; ++c) {
          ld_chunk<CI>(w + ib + c * cstride, wl + 1 + c * CI);
          if (first) {
#pragma unroll
            for (int r = 0; r < CI; ++r) vl[1 + c * CI + r] = 0.f;
          } else {
            ld_chunk<CI>(vold + ib + c * cstride, vl + 1 + c * CI);
          }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int i = q ? N1 - 1 : 0;
          wl[i] = gi[i] >= 0 ? w[gi[i]] : 0.f;
          vl[i] = (gi[i] >= 0 && !first) ? vold[gi[i]] : 0.f;
        }
      } else {
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          wl[i] = gi[i] >= 0 ? w[gi[i]] : 0.f;
          vl[i] = (gi[i] >= 0 && !first) ? vold[gi[i]] : 0.f;
        }
      }
#pragma unroll
      for (int i = 0; i < N1; ++i) u[i] = first ? wl[i] : wl[i] + beta * vl[i];
      if (irow) {
#pragma unroll
        for (int c = 0; c < M / CI; ++c) st_chunk<CI>(vnew + ib + c * cstride, u + 1 + c * CI);
        if (own & 1u) vnew[gi[0]] = u[0];
        if ((own >> (N1 - 1)) & 1u) vnew[gi[N1 - 1]] = u[N1 - 1];
      } else {
#pragma unroll
        for (int i = 0; i < N1; ++i)
          if ((own >> i) & 1u) vnew[gi[i]] = u[i];
      }
    }
    line_op_f32<N1, NF>(Cg.D, fl, active, le < EPL ? le : 0, t, X, Y, u, Lu);
    if (active) {
      // contribution slots from the descriptor again (an L1 hit): no index registers live across the operator
      int gi[N1], zi[N1];
      unsigned own;
      compact_line<N1>(V, e, t, V.desc[3 * e], V.desc[3 * e + 1], V.desc[3 * e + 2], gi, zi, own);
      if (irow) {
#pragma unroll
        for (int c = 0; c < M / CI; ++c) st_chunk<CI>(zc + ib + c * cstride, Lu + 1 + c * CI);
        if (zi[0] >= 0) zc[zi[0]] = Lu[0];
        if (zi[N1 - 1] >= 0) zc[zi[N1 - 1]] = Lu[N1 - 1];
      } else {
#pragma unroll
        for (int i = 0; i < N1; ++i)
          if (zi[i] >= 0) zc[zi[i]] = Lu[i];
      }
#pragma unroll
      for (int i = 0; i < N1; ++i) pa += u[i] * Lu[i];
    }
    line_sync<N1>();  // the next pass reuses X and Y (warp-synchronous: each warp runs through the passes on its own)
  }
  const float acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, float>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->vz = tot[0];
    S->alpha = S->num / tot[0];
    S->alpha32 = (float)S->alpha;
  }
}

// FP64 form: the even-odd FP64 line operator of pcg_apply_fused_eo (line_op_f64, factors in the element-local
// layout) with the compact gathers and slot stores of pcg_apply_compact_f32.
template <int N1, int NF>
__global__ void __launch_bounds__(kRedThreads, 2) pcg_apply_compact_f64(const double* __restrict__ w,
                                                                        const double* __restrict__ vold,
                                                                        double* __restrict__ vnew, CompactView V,
                                                                        const double* __restrict__ fac,
                                                                        double* __restrict__ zc, EOPair<N1> Tg,
                                                                        CGScalars* S, double* __restrict__ partial,
                                                                        unsigned int* __restrict__ ticket) {
  if (S->done) return;
  constexpr int M = N1 - 2, NN = N1 * N1;
  constexpr int EPL = line_epb<N1>();
  constexpr int LS = N1 + 1;
  constexpr int CI = chunk_of<M>();
  __shared__ EOPair<N1> T;
  __shared__ double X[EPL * N1 * LS];
  __shared__ double Y[EPL * N1 * LS];
  eo_copy_tables<N1>(Tg, T);
  __syncthreads();
  const int nEl = V.nEl;
  const int le = threadIdx.x / N1, t = threadIdx.x - le * N1;
  const bool first = S->iter == 0;
  const double beta = first ? 0.0 : S->beta;
  const int ngroups = (nEl + EPL - 1) / EPL;
  const bool irow = t > 0 && t < N1 - 1;
  double pa = 0.0;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int e = g * EPL + le;
    const bool active = le < EPL && e < nEl;
    double u[N1], Lu[N1];
    int ib = 0, cstride = 0;
    if (active) {
      int gi[N1], zi[N1];
      unsigned own;
      compact_line<N1>(V, e, t, V.desc[3 * e], V.desc[3 * e + 1], V.desc[3 * e + 2], gi, zi, own);
      double wl[N1], vl[N1];
      if (irow) {
        const int ne = min(EPL, nEl - g * EPL);
        ib = interior_index<N1>(e, 0, t - 1, nEl);
        cstride = ne * M * CI;
#pragma unroll
        for (int c = 0; c < M / CI; ++c) {
          ld_chunk<CI>(w + ib + c * cstride, wl + 1 + c * CI);
          if (first) {
#pragma unroll
            for (int r = 0; r < CI; ++r) vl[1 + c * CI + r] = 0.0;
          } else {
            ld_chunk<CI>(vold + ib + c * cstride, vl + 1 + c * CI);
          }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int i = q ? N1 - 1 : 0;
          wl[i] = gi[i] >= 0 ? w[gi[i]] : 0.0;
          vl[i] = (gi[i] >= 0 && !first) ? vold[gi[i]] : 0.0;
        }
      } else {
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          wl[i] = gi[i] >= 0 ? w[gi[i]] : 0.0;
          vl[i] = (gi[i] >= 0 && !first) ? vold[gi[i]] : 0.0;
        }
      }
#pragma unroll
      for (int i = 0; i < N1; ++i) u[i] = first ? wl[i] : wl[i] + beta * vl[i];
      if (irow) {
#pragma unroll
        for (int c = 0; c < M / CI; ++c) st_chunk<CI>(vnew + ib + c * cstride, u + 1 + c * CI);
        if (own & 1u) vnew[gi[0]] = u[0];
        if ((own >> (N1 - 1)) & 1u) vnew[gi[N1 - 1]] = u[N1 - 1];
      } else {
#pragma unroll
        for (int i = 0; i < N1; ++i)
          if ((own >> i) & 1u) vnew[gi[i]] = u[i];
      }
    }
    line_op_f64<N1, NF>(T, fac + (size_t)(active ? e : 0) * NF * NN + (size_t)N1 * t, active, le < EPL ? le : 0, t, X,
                        Y, u, Lu);
    if (active) {
      int gi[N1], zi[N1];
      unsigned own;
      compact_line<N1>(V, e, t, V.desc[3 * e], V.desc[3 * e + 1], V.desc[3 * e + 2], gi, zi, own);
      if (irow) {
#pragma unroll
        for (int c = 0; c < M / CI; ++c) st_chunk<CI>(zc + ib + c * cstride, Lu + 1 + c * CI);
        if (zi[0] >= 0) zc[zi[0]] = Lu[0];
        if (zi[N1 - 1] >= 0) zc[zi[N1 - 1]] = Lu[N1 - 1];
      } else {
#pragma unroll
        for (int i = 0; i < N1; ++i)
          if (zi[i] >= 0) zc[zi[i]] = Lu[i];
      }
#pragma unroll
      for (int i = 0; i < N1; ++i) pa += u[i] * Lu[i];
    }
  }
  const double acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, double>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->vz = tot[0];
    S->alpha = S->num / tot[0];
    S->alpha32 = (float)S->alpha;
  }
}

// Assembled z at compact node m from the contribution space (see the file header for the sums).
template <int N1, typename R>
__device__ __forceinline__ R compact_z(const CompactView& V, const R* __restrict__ zc, int m) {
  constexpr int M = N1 - 2;
  if (m < V.nInt) return zc[m];
  int q = m - V.nInt;
  const int nEM = (V.nE2 + V.nE1) * M;
  if (q < nEM) {
    const int id = q / M, k = q - id * M;
    const int b = V.nInt + 2 * id * M + k;
    return id < V.nE2 ? zc[b] + zc[b + M] : zc[b];
  }
  q -= nEM;
  if (q >= V.nC) return R(0);  // padding
  const R* c = zc + V.nInt + 2 * nEM;
  R s = 0;
  for (int k = V.coff[q], k1 = V.coff[q + 1]; k < k1; ++k) s += c[k];
  return s;
}

// four consecutive nodes (16-byte aligned for FP32, two 16-byte halves for FP64)
template <typename R>
struct Q4 {
  R x, y, z, w;
};
__device__ __forceinline__ Q4<float> ld4(const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Q4<double> ld4(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(float* p, const Q4<float>& q) {
  *reinterpret_cast<float4*>(p) = make_float4(q.x, q.y, q.z, q.w);
}
__device__ __forceinline__ void st4(double* p, const Q4<double>& q) {
  reinterpret_cast<double2*>(p)[0] = make_double2(q.x, q.y);
  reinterpret_cast<double2*>(p)[1] = make_double2(q.z, q.w);
}

// a = num/<v,z>; u += a v, r -= a z, w = dinv r over groups of 4 nodes of the compact vectors (z assembled on the
// fly from the contribution space), partial sums of <r,w> and <r,r>, then the end-of-iteration scalar step.
template <int N1, typename R>
__global__ void __launch_bounds__(kRedThreads) pcg_update_compact(R* __restrict__ u, R* __restrict__ r,
                                                                  R* __restrict__ w, const R* __restrict__ v,
                                                                  const R* __restrict__ zc,
                                                                  const R* __restrict__ dinv, CompactView V,
                                                                  CGScalars* S, double* __restrict__ partial,
                                                                  unsigned int* __restrict__ ticket) {
  if (S->done) return;
  const R a = sizeof(R) == 4 ? (R)S->alpha32 : (R)S->alpha;
  R prw = 0, prr = 0;
  const int nq = V.ngp / 4, nqi = V.nInt / 4, stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const Q4<R> one{1, 1, 1, 1};
  auto update = [&](int q, const Q4<R>& uu, const Q4<R>& vv, const Q4<R>& rr, const Q4<R>& dd, const Q4<R>& zz) {
    Q4<R> uo, ro, wo;
    uo.x = uu.x + a * vv.x;
    uo.y = uu.y + a * vv.y;
    uo.z = uu.z + a * vv.z;
    uo.w = uu.w + a * vv.w;
    ro.x = rr.x - a * zz.x;
    ro.y = rr.y - a * zz.y;
    ro.z = rr.z - a * zz.z;
    ro.w = rr.w - a * zz.w;
    wo.x = dinv ? ro.x * dd.x : ro.x;
    wo.y = dinv ? ro.y * dd.y : ro.y;
    wo.z = dinv ? ro.z * dd.z : ro.z;
    wo.w = dinv ? ro.w * dd.w : ro.w;
    prw += ro.x * wo.x + ro.y * wo.y + ro.z * wo.z + ro.w * wo.w;
    prr += ro.x * ro.x + ro.y * ro.y + ro.z * ro.z + ro.w * ro.w;
    st4(u + 4 * q, uo);
    st4(r + 4 * q, ro);
    st4(w + 4 * q, wo);
  };
  // interior groups: plain streams, U groups per thread with every load issued before any use (FP64: one, the
  // registers of two would cost occupancy)
  constexpr int U = sizeof(R) == 4 ? 2 : 1;
  for (int q0 = tid; q0 < nqi; q0 += U * stride) {
    Q4<R> uu[U], vv[U], rr[U], dd[U], zz[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int q = q0 + k * stride;
      if (q >= nqi) continue;
      uu[k] = ld4(u + 4 * q);
      vv[k] = ld4(v + 4 * q);
      rr[k] = ld4(r + 4 * q);
      dd[k] = dinv ? ld4(dinv + 4 * q) : one;
      zz[k] = ld4(zc + 4 * q);
    }
#pragma unroll
    for (int k = 0; k < U; ++k)
      if (q0 + k * stride < nqi) update(q0 + k * stride, uu[k], vv[k], rr[k], dd[k], zz[k]);
  }
  // shared-node groups (and the group straddling the interior's end): z assembled from the contribution slots
  for (int q = nqi + tid; q < nq; q += stride) {
    const Q4<R> uu = ld4(u + 4 * q), vv = ld4(v + 4 * q), rr = ld4(r + 4 * q);
    const Q4<R> dd = dinv ? ld4(dinv + 4 * q) : one;
    Q4<R> zz;
    zz.x = compact_z<N1>(V, zc, 4 * q);
    zz.y = compact_z<N1>(V, zc, 4 * q + 1);
    zz.z = compact_z<N1>(V, zc, 4 * q + 2);
    zz.w = compact_z<N1>(V, zc, 4 * q + 3);
    update(q, uu, vv, rr, dd, zz);
  }
  const R acc[2] = {prw, prr};
  double tot[2];
  if (grid_sums_last<2, R>(acc, partial, ticket, tot) && threadIdx.x == 0) pcg_end_iteration(S, tot[0], tot[1]);
}

// out[cl[n]] = assembled z at unknown n (out zero elsewhere: the masked L-vector of Mask(GlobalSum(L v)))
template <int N1, typename R>
__global__ void compact_assemble(double* __restrict__ out, const R* __restrict__ zc, const int* __restrict__ cl,
                                 int ng, CompactView V) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < ng; n += gridDim.x * blockDim.x)
    out[cl[n]] = (double)compact_z<N1>(V, zc, n);
}

// y[n] = (R) x[cl[n]] (the unknown's primary copy in the masked FP64 L-vector); padding zero
template <typename R>
__global__ void compact_gather(R* __restrict__ y, const double* __restrict__ x, const int* __restrict__ cl, int ng,
                               int ngp) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < ngp; n += gridDim.x * blockDim.x)
    y[n] = n < ng ? (R)x[cl[n]] : R(0);
}

// x[cl[n]] += y[n]: a correction on the compact layout added to the masked FP64 iterate at the primary copies
template <typename R>
__global__ void compact_scatter_add(double* __restrict__ x, const R* __restrict__ y, const int* __restrict__ cl,
                                    int ng) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < ng; n += gridDim.x * blockDim.x) x[cl[n]] += (double)y[n];
}
