// Host-side set-up of libselfgpu: context and error handling, nodal storage, the structured
// quadrilateral mesh with its edge table and mapped geometry, and the bathymetry gradient.
// These are the Build procedures of the reference (NodalStorage_2D%Build, QuadMesh%LoadDefaultMesh,
// MappedGeometry_2D%Build, ShallowWater%CalculateBathymetryGradient) that produce the arrays the
// GPU path consumes.  They run once, on the host, in FP64.
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <string>
#include <sstream>
#include <vector>

#include "internal.hpp"

#include <map>

namespace selfgpu {

// Page-locked, mapped host blocks handed out by self_host_alloc (start -> size).
namespace {
std::mutex g_host_mu;
std::map<uintptr_t, size_t> g_host_blocks;
}  // namespace

void host_blocks_add(const void* p, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_blocks[reinterpret_cast<uintptr_t>(p)] = bytes;
}

void host_blocks_remove(const void* p) {
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_blocks.erase(reinterpret_cast<uintptr_t>(p));
}

void* mapped_host(const void* p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_blocks.upper_bound(a);
    if (it == g_host_blocks.begin()) return nullptr;
    --it;
    if (a < it->first || a + bytes > it->first + it->second) return nullptr;
  }
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, const_cast<void*>(p), 0) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return d;
}

}  // namespace selfgpu

namespace selfgpu {

static std::mutex g_err_mu;
static std::string g_err;

int set_error(self_ctx* ctx, int status, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->last_error = buf;
  set_global_error(buf);
  return status;
}

void set_global_error(const char* msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err = msg;
}

// ------------------------------------------------------------------ polynomial tools
namespace {

const double kPi = 3.14159265358979323846;

// Legendre P_n and P_n' by the three-term recurrence.
void legendre(int n, double x, double& p, double& dp) {
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (n == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    double d2 = d0 + (2.0 * k - 1.0) * p1;
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  p = p1;
  dp = d1;
}

// Roots of P_{N+1} (Gauss) or of (1-x^2) P_N' (Gauss-Lobatto) by Newton from Chebyshev-type guesses.
void quadrature(int N, int quad, std::vector<double>& x, std::vector<double>& w) {
  x.assign(N + 1, 0.0);
  w.assign(N + 1, 0.0);
  if (quad == SELF_GAUSS) {
    if (N == 0) {
      w[0] = 2.0;
      return;
    }
    for (int j = 0; j <= N / 2; ++j) {
      double r = -std::cos((2.0 * j + 1.0) * kPi / (2.0 * N + 2.0));
      for (int it = 0; it < 100; ++it) {
        double p, dp;
        legendre(N + 1, r, p, dp);
        double d = -p / dp;
        r += d;
        if (std::fabs(d) < 1e-16) break;
      }
      double p, dp;
      legendre(N + 1, r, p, dp);
      x[j] = r;
      x[N - j] = -r;
      w[j] = w[N - j] = 2.0 / ((1.0 - r * r) * dp * dp);
    }
    if (N % 2 == 0) {
      double p, dp;
      legendre(N + 1, 0.0, p, dp);
      x[N / 2] = 0.0;
      w[N / 2] = 2.0 / (dp * dp);
    }
  } else {
    x[0] = -1.0;
    x[N] = 1.0;
    w[0] = w[N] = 2.0 / (N * (N + 1.0));
    for (int j = 1; j <= (N - 1) / 2; ++j) {
      double r = -std::cos(kPi * j / N);
      for (int it = 0; it < 100; ++it) {
        // q = P_{N+1} - P_{N-1} vanishes at the interior Lobatto points; q' = (2N+1) P_N
        double pn, dpn, pm, dpm, pp, dpp;
        legendre(N - 1, r, pm, dpm);
        legendre(N, r, pn, dpn);
        legendre(N + 1, r, pp, dpp);
        double d = -(pp - pm) / ((2.0 * N + 1.0) * pn);
        r += d;
        if (std::fabs(d) < 1e-16) break;
      }
      double pn, dpn;
      legendre(N, r, pn, dpn);
      x[j] = r;
      x[N - j] = -r;
      w[j] = w[N - j] = 2.0 / (N * (N + 1.0) * pn * pn);
    }
    if (N % 2 == 0) {
      double pn, dpn;
      legendre(N, 0.0, pn, dpn);
      x[N / 2] = 0.0;
      w[N / 2] = 2.0 / (N * (N + 1.0) * pn * pn);
    }
  }
}

struct Interp1D {
  int N;
  std::vector<double> x, bw;
  void build(const std::vector<double>& nodes) {
    x = nodes;
    N = (int)x.size() - 1;
    bw.assign(N + 1, 1.0);
    for (int j = 0; j <= N; ++j)
      for (int k = 0; k <= N; ++k)
        if (k != j) bw[j] *= (x[j] - x[k]);
    for (int j = 0; j <= N; ++j) bw[j] = 1.0 / bw[j];
  }
  // Lagrange basis values at xe
  void basis(double xe, double* l) const {
    for (int j = 0; j <= N; ++j)
      if (xe == x[j]) {
        for (int k = 0; k <= N; ++k) l[k] = (k == j) ? 1.0 : 0.0;
        return;
      }
    double s = 0.0;
    for (int j = 0; j <= N; ++j) {
      l[j] = bw[j] / (xe - x[j]);
      s += l[j];
    }
    for (int j = 0; j <= N; ++j) l[j] /= s;
  }
  // derivative of the Lagrange basis at xe
  void dbasis(double xe, double* dl) const {
    for (int i = 0; i <= N; ++i)
      if (xe == x[i]) {  // at a node: the row of the collocation derivative matrix
        std::vector<double> D((N + 1) * (N + 1));
        dmatrix(D.data());
        for (int j = 0; j <= N; ++j) dl[j] = D[i + j * (N + 1)];
        return;
      }
    std::vector<double> l(N + 1);
    basis(xe, l.data());
    double s = 0.0;
    for (int j = 0; j <= N; ++j) s += bw[j] / (xe - x[j]);
    // l_j'(x) = l_j(x) * [ 1/(x - x_j) ... ] via the barycentric identity
    double t = 0.0;
    for (int j = 0; j <= N; ++j) t += bw[j] / ((xe - x[j]) * (xe - x[j]));
    for (int j = 0; j <= N; ++j) dl[j] = l[j] * (t / s - 1.0 / (xe - x[j]));
  }
  // collocation derivative matrix D(i,j) = l_j'(x_i), column major
  void dmatrix(double* D) const {
    int n = N + 1;
    for (int i = 0; i < n; ++i) {
      double diag = 0.0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        D[i + j * n] = (bw[j] / bw[i]) / (x[i] - x[j]);
        diag -= D[i + j * n];
      }
      D[i + i * n] = diag;
    }
  }
};

}  // namespace
}  // namespace selfgpu

using namespace selfgpu;

extern "C" {

const char* self_status_string(int s) {
  switch (s) {
    case SELF_OK: return "ok";
    case SELF_ERR_INVALID: return "invalid argument";
    case SELF_ERR_CUDA: return "CUDA error";
    case SELF_ERR_ALLOC: return "allocation failed";
    case SELF_ERR_UNSUPPORTED: return "unsupported option";
    case SELF_ERR_TIMEOUT: return "device wait timed out";
    case SELF_ERR_NOT_CONVERGED: return "solver did not converge";
    case SELF_ERR_NONFINITE: return "non-finite value";
    default: return "unknown status";
  }
}

int self_last_error(const self_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return SELF_ERR_INVALID;
  std::string s;
  if (ctx) {
    s = ctx->last_error;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    s = g_err;
  }
  snprintf(buf, len, "%s", s.c_str());
  return SELF_OK;
}

int self_ctx_create(int device, self_ctx** out) {
  if (!out) return SELF_ERR_INVALID;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return set_error(nullptr, SELF_ERR_CUDA, "no CUDA device available: %s", cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return set_error(nullptr, SELF_ERR_INVALID, "device %d out of range", device);
  auto* c = new (std::nothrow) self_ctx();
  if (!c) return SELF_ERR_ALLOC;
  c->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete c;
    return set_error(nullptr, SELF_ERR_CUDA, "context set-up failed: %s", cudaGetErrorString(e));
  }
  *out = c;
  return SELF_OK;
}

int self_ctx_destroy(self_ctx* ctx) {
  if (!ctx) return SELF_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->flush_buf) cudaFree(ctx->flush_buf);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SELF_OK;
}

int self_ctx_synchronize(self_ctx* ctx) {
  if (!ctx) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return SELF_OK;
}

long long self_ctx_kernel_launches(const self_ctx* ctx) { return ctx ? ctx->launches.load() : 0; }

int self_ctx_timer_start(self_ctx* ctx) {
  if (!ctx) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (!ctx->ev0) SELF_CUDA_TRY(ctx, cudaEventCreate(&ctx->ev0));
  if (!ctx->ev1) SELF_CUDA_TRY(ctx, cudaEventCreate(&ctx->ev1));
  SELF_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  return SELF_OK;
}

int self_ctx_timer_stop(self_ctx* ctx, double* ms) {
  if (!ctx || !ms || !ctx->ev0) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
  float f = 0.f;
  SELF_CUDA_TRY(ctx, cudaEventElapsedTime(&f, ctx->ev0, ctx->ev1));
  *ms = f;
  return SELF_OK;
}

int self_ctx_query(self_ctx* ctx) {
  if (!ctx) return SELF_ERR_INVALID;
  cudaError_t e = cudaStreamQuery(ctx->stream);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return set_error(ctx, SELF_ERR_CUDA, "stream query: %s", cudaGetErrorString(e));
}

int self_ctx_host_loop(self_ctx* ctx, int host_loop) {
  if (!ctx) return SELF_ERR_INVALID;
  ctx->host_loop = host_loop ? 1 : 0;
  return SELF_OK;
}

int self_ctx_flush_l2(self_ctx* ctx, size_t bytes) {
  if (!ctx) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (ctx->flush_bytes < bytes) {
    if (ctx->flush_buf) cudaFree(ctx->flush_buf);
    ctx->flush_buf = nullptr;
    ctx->flush_bytes = 0;
    SELF_CUDA_TRY(ctx, cudaMalloc(&ctx->flush_buf, bytes));
    ctx->flush_bytes = bytes;
  }
  SELF_CUDA_TRY(ctx, cudaMemsetAsync(ctx->flush_buf, (int)(ctx->launches.load() & 0xff), bytes, ctx->stream));
  return SELF_OK;
}

int self_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return SELF_ERR_INVALID;
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
  if (e != cudaSuccess) return set_error(nullptr, SELF_ERR_ALLOC, "cudaHostAlloc: %s", cudaGetErrorString(e));
  selfgpu::host_blocks_add(*ptr, bytes);
  return SELF_OK;
}

int self_host_free(void* ptr) {
  if (ptr) {
    selfgpu::host_blocks_remove(ptr);
    cudaFreeHost(ptr);
  }
  return SELF_OK;
}

int self_nodal_build(int N, int quad, int form, double* nodes, double* qw, double* dmatS, double* dmatP,
                     double* lW, double* lE, double* lS, double* lN) {
  if (N < 1 || N > 15) return set_error(nullptr, SELF_ERR_INVALID, "polynomial degree %d outside 1..15", N);
  if (quad != SELF_GAUSS && quad != SELF_GAUSS_LOBATTO) return set_error(nullptr, SELF_ERR_INVALID, "quadrature");
  std::vector<double> x, w;
  quadrature(N, quad, x, w);
  Interp1D I;
  I.build(x);
  const int n = N + 1;
  std::vector<double> D(n * n);
  I.dmatrix(D.data());
  for (int i = 0; i < n; ++i) {
    nodes[i] = x[i];
    qw[i] = w[i];
  }
  I.basis(-1.0, lW);
  I.basis(1.0, lE);
  I.basis(-1.0, lS);
  I.basis(1.0, lN);
  if (form == SELF_CG) {
    for (int k = 0; k < n * n; ++k) dmatS[k] = dmatP[k] = D[k];
  } else if (form == SELF_DG) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) dmatS[i + j * n] = dmatP[i + j * n] = -D[j + i * n] * w[j] / w[i];
  } else {
    return set_error(nullptr, SELF_ERR_INVALID, "form must be SELF_DG or SELF_CG");
  }
  return SELF_OK;
}

int self_mesh_counts(int nx, int ny, int px, int py, int* nEl, int* nEdges, int* nNodes) {
  if (nx < 1 || ny < 1 || (px && nx < 3) || (py && ny < 3))
    return set_error(nullptr, SELF_ERR_INVALID, "mesh %dx%d invalid (periodic directions need >= 3)", nx, ny);
  *nEl = nx * ny;
  *nNodes = (px ? nx : nx + 1) * (py ? ny : ny + 1);
  *nEdges = (px ? nx : nx + 1) * ny + nx * (py ? ny : ny + 1);
  return SELF_OK;
}

int self_mesh_build(int nx, int ny, int px, int py, int N, int quad, double warp, double xscale, double yscale,
                    int bflag, int* edges, int* elemNodes, int* nodeType, int* n2e_ptr, int* n2e_elem,
                    int* n2e_local, double* X, double* Y, double* dxds, double* dxdp, double* dyds, double* dydp,
                    double* J, double* nhx, double* nhy, double* nlen, double* bx, double* by) {
  int nEl, nEdges, nNodes;
  int rc = self_mesh_counts(nx, ny, px, py, &nEl, &nEdges, &nNodes);
  if (rc) return rc;
  if (N < 1 || N > 15) return set_error(nullptr, SELF_ERR_INVALID, "polynomial degree %d outside 1..15", N);
  const int n = N + 1;
  const int NX = px ? nx : nx + 1;
  auto node_id = [&](int ix, int iy) {  // 0-based corner grid -> 1-based node ID
    if (px) ix %= nx;
    if (py) iy %= ny;
    return 1 + ix + iy * NX;
  };
  std::vector<double> xq, wq;
  quadrature(N, quad, xq, wq);
  Interp1D I;
  I.build(xq);
  std::vector<double> D(n * n), lm(n), lp(n), dlm(n), dlp(n);
  I.dmatrix(D.data());
  I.basis(-1.0, lm.data());
  I.basis(1.0, lp.data());
  I.dbasis(-1.0, dlm.data());
  I.dbasis(1.0, dlp.data());

  auto map_point = [&](double ux, double uy, double& ox, double& oy) {
    double s = warp * std::sin(2.0 * kPi * ux) * std::sin(2.0 * kPi * uy);
    ox = xscale * (ux + s);
    oy = yscale * (uy + s);
  };
  for (int k = 0; k < nNodes; ++k) nodeType[k] = 0;
  std::vector<double> xs(n * n), ys(n * n);
  for (int iy = 0; iy < ny; ++iy)
    for (int ix = 0; ix < nx; ++ix) {
      const int e = ix + iy * nx;
      elemNodes[4 * e + 0] = node_id(ix, iy);
      elemNodes[4 * e + 1] = node_id(ix + 1, iy);
      elemNodes[4 * e + 2] = node_id(ix + 1, iy + 1);
      elemNodes[4 * e + 3] = node_id(ix, iy + 1);
      const double x0 = (double)ix / nx, x1 = (double)(ix + 1) / nx;
      const double y0 = (double)iy / ny, y1 = (double)(iy + 1) / ny;
      auto unit_point = [&](double s, double p, double& ux, double& uy) {
        ux = x0 + (x1 - x0) * 0.5 * (s + 1.0);
        uy = y0 + (y1 - y0) * 0.5 * (p + 1.0);
      };
      const size_t o = (size_t)n * n * e;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double ux, uy;
          unit_point(xq[i], xq[j], ux, uy);
          map_point(ux, uy, X[o + i + n * j], Y[o + i + n * j]);
        }
      // covariant metrics from the derivative of the degree-N interpolant of the node positions
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double a = 0, b = 0, c = 0, d = 0;
          for (int k = 0; k < n; ++k) {
            a += D[i + k * n] * X[o + k + n * j];
            c += D[i + k * n] * Y[o + k + n * j];
            b += D[j + k * n] * X[o + i + n * k];
            d += D[j + k * n] * Y[o + i + n * k];
          }
          dxds[o + i + n * j] = a;
          dxdp[o + i + n * j] = b;
          dyds[o + i + n * j] = c;
          dydp[o + i + n * j] = d;
          J[o + i + n * j] = a * d - b * c;
        }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) xs[i + n * j] = dxds[o + i + n * j], ys[i + n * j] = dyds[o + i + n * j];
      // boundary points, boundary metrics and outward unit normals
      for (int side = 0; side < 4; ++side)
        for (int k = 0; k < n; ++k) {
          double s = 0, p = 0;
          double a = 0, b = 0, c = 0, d = 0;  // dxds dxdp dyds dydp at the boundary point
          if (side == 0 || side == 2) {
            p = (side == 0) ? -1.0 : 1.0;
            s = xq[k];
            const double* l = (side == 0) ? lm.data() : lp.data();
            const double* dl = (side == 0) ? dlm.data() : dlp.data();
            for (int j = 0; j < n; ++j) {
              a += l[j] * xs[k + n * j];
              c += l[j] * ys[k + n * j];
              b += dl[j] * X[o + k + n * j];
              d += dl[j] * Y[o + k + n * j];
            }
          } else {
            s = (side == 1) ? 1.0 : -1.0;
            p = xq[k];
            const double* l = (side == 1) ? lp.data() : lm.data();
            const double* dl = (side == 1) ? dlp.data() : dlm.data();
            for (int i = 0; i < n; ++i) {
              a += dl[i] * X[o + i + n * k];
              c += dl[i] * Y[o + i + n * k];
            }
            // d/dp along the side: interpolate the p-derivative of the node positions to s = +-1
            for (int i = 0; i < n; ++i) {
              double xp = 0, yp = 0;
              for (int m = 0; m < n; ++m) {
                xp += D[k + m * n] * X[o + i + n * m];
                yp += D[k + m * n] * Y[o + i + n * m];
              }
              b += l[i] * xp;
              d += l[i] * yp;
            }
          }
          double ux, uy;
          unit_point(s, p, ux, uy);
          const size_t ib = (size_t)k + n * (side + 4 * (size_t)e);
          map_point(ux, uy, bx[ib], by[ib]);
          double Jb = a * d - b * c;
          double sg = Jb > 0 ? 1.0 : -1.0;
          double d0, d1;
          switch (side) {
            case 0: d0 = sg * c; d1 = -sg * a; break;   // -(-dyds, dxds)
            case 2: d0 = -sg * c; d1 = sg * a; break;   //  (-dyds, dxds)
            case 3: d0 = -sg * d; d1 = sg * b; break;   // -(dydp, -dxdp)
            default: d0 = sg * d; d1 = -sg * b; break;  //  (dydp, -dxdp)
          }
          double len = std::sqrt(d0 * d0 + d1 * d1);
          nhx[ib] = d0 / len;
          nhy[ib] = d1 / len;
          nlen[ib] = len;
        }
    }
  // Edge table in order of first appearance (element order, sides S,E,N,W), as ConstructEdges.
  // Structured edge keys: horizontal edge below row iy at column ix; vertical edge left of column ix.
  const int HY = py ? ny : ny + 1, VX = px ? nx : nx + 1;
  std::vector<int> hid((size_t)nx * HY, 0), vid((size_t)VX * ny, 0);
  static const int emap[2][4] = {{0, 1, 3, 0}, {1, 2, 2, 3}};  // local corners (0-based) per side
  int ne = 0;
  for (int iy = 0; iy < ny; ++iy)
    for (int ix = 0; ix < nx; ++ix) {
      const int e = ix + iy * nx;
      for (int k = 0; k < 4; ++k) {
        int* slot;
        switch (k) {
          case 0: slot = &hid[ix + (size_t)nx * iy]; break;
          case 2: slot = &hid[ix + (size_t)nx * ((iy + 1) % HY)]; break;
          case 1: slot = &vid[((ix + 1) % VX) + (size_t)VX * iy]; break;
          default: slot = &vid[ix + (size_t)VX * iy]; break;
        }
        int startID = elemNodes[4 * e + emap[0][k]];
        if (*slot == 0) {
          *slot = ++ne;
          int* E = edges + 6 * (ne - 1);
          E[0] = e + 1;
          E[1] = k + 1;
          E[2] = bflag;
          E[3] = 0;
          E[4] = 1;
          E[5] = 1;
        } else {
          int* E = edges + 6 * (*slot - 1);
          int n1 = elemNodes[4 * (E[0] - 1) + emap[0][E[1] - 1]];
          E[2] = e + 1;
          E[3] = (startID == n1) ? (k + 1) : -(k + 1);
          if (E[3] < 0) {
            E[4] = N - 1;
            E[5] = -1;
          }
        }
      }
    }
  if (ne != nEdges) return set_error(nullptr, SELF_ERR_INVALID, "edge count mismatch %d != %d", ne, nEdges);
  for (int k = 0; k < nEdges; ++k) {
    const int* E = edges + 6 * k;
    if (E[2] < 0) {
      int e = E[0] - 1, s = E[1] - 1;
      nodeType[elemNodes[4 * e + emap[0][s]] - 1] = E[2];
      nodeType[elemNodes[4 * e + emap[1][s]] - 1] = E[2];
    }
  }
  // corner node -> element lists in element order (tail insertion)
  std::vector<int> cnt(nNodes + 1, 0);
  for (int e = 0; e < nEl; ++e)
    for (int c = 0; c < 4; ++c) cnt[elemNodes[4 * e + c]]++;
  n2e_ptr[0] = 0;
  for (int i = 0; i < nNodes; ++i) n2e_ptr[i + 1] = n2e_ptr[i] + cnt[i + 1];
  std::vector<int> pos(n2e_ptr, n2e_ptr + nNodes);
  for (int e = 0; e < nEl; ++e)
    for (int c = 0; c < 4; ++c) {
      int nd = elemNodes[4 * e + c] - 1;
      n2e_elem[pos[nd]] = e + 1;
      n2e_local[pos[nd]] = c + 1;
      pos[nd]++;
    }
  return SELF_OK;
}

// ------------------------------------------------------------------------------------------------ ISM-V2 meshes
// SpecMesh ISM-V2 files (ReadSpecMeshFile_QuadMesh, QuadMeshClass.f90:2100-2475): corner nodes, an edge list
// (not used: the edges are rebuilt from the elements as ConstructEdges does), and per element 4 corner node IDs,
// 4 side kinds (0 straight interior side, 1 boundary curve given by its points at the Chebyshev-Gauss-Lobatto
// nodes of the file's geometry degree) and 4 side names (boundary condition).  The element geometry is the
// transfinite (Coons) blend of the 4 side curves with its analytic covariant metrics (Build_MappedGeometry_2D,
// MappedGeometryClass_2D.f90:105-144, 536-710).
namespace {

struct IsmMesh {
  int nNodes = 0, nEdges = 0, nElems = 0, gdeg = 1;
  std::vector<double> px, py;           // corner nodes
  std::vector<int> corner;              // 4 per element, 1-based
  std::vector<int> kind;                // 4 per element
  std::vector<std::vector<double>> cx, cy;
  std::vector<int> bc;                  // boundary flag per element side (1 = interior / unnamed)
};

int ism_flag(const std::string& w) {
  static const std::pair<const char*, int> names[] = {
      {"NO_NORMAL_FLOW", -100}, {"NEUMANN", -100},  {"RADIATION", -101},          {"PRESCRIBED", -102},
      {"InflowOne", -103},      {"InflowTwo", -104}, {"DIRICHLET", -200},          {"HOMOGENEOUS_NEUMANN", -201},
      {"ROBIN", -202},          {"ROBIN_FORCED", -204}, {"NEUMANN_WALL", -206}};
  for (const auto& nm : names)
    if (w == nm.first) return nm.second;
  return 1;
}

int ism_read(const char* path, IsmMesh& m, bool header_only) {
  FILE* fp = fopen(path, "r");
  if (!fp) return set_error(nullptr, SELF_ERR_INVALID, "cannot open mesh file %s", path);
  std::string text;
  char chunk[65536];
  size_t got;
  while ((got = fread(chunk, 1, sizeof(chunk), fp)) > 0) text.append(chunk, got);
  fclose(fp);
  // line-oriented: the side-name line is read whole, everything else as blank-separated numbers
  std::vector<std::string> lines;
  {
    size_t a = 0;
    while (a < text.size()) {
      size_t b = text.find('\n', a);
      if (b == std::string::npos) b = text.size();
      lines.emplace_back(text.substr(a, b - a));
      a = b + 1;
    }
  }
  size_t li = 1;  // line 0: version tag
  auto numbers = [&](size_t k, std::vector<double>& out) {
    out.clear();
    if (k >= lines.size()) return false;
    const char* c = lines[k].c_str();
    char* end;
    for (;;) {
      while (*c == ' ' || *c == '\t' || *c == '\r') ++c;
      if (!*c) break;
      const double v = strtod(c, &end);
      if (end == c) return false;
      out.push_back(v);
      c = end;
    }
    return true;
  };
  std::vector<double> v;
  if (!numbers(li++, v) || v.size() < 4) return set_error(nullptr, SELF_ERR_INVALID, "%s: bad ISM header", path);
  m.nNodes = (int)v[0];
  m.nEdges = (int)v[1];
  m.nElems = (int)v[2];
  m.gdeg = (int)v[3];
  if (m.nNodes < 4 || m.nElems < 1 || m.nEdges < 4 || m.gdeg < 1)
    return set_error(nullptr, SELF_ERR_INVALID, "%s: bad ISM counts", path);
  if (header_only) return SELF_OK;
  auto fail = [&](const char* what) { return set_error(nullptr, SELF_ERR_INVALID, "%s: %s", path, what); };
  m.px.resize(m.nNodes);
  m.py.resize(m.nNodes);
  for (int k = 0; k < m.nNodes; ++k) {
    if (!numbers(li++, v) || v.size() < 2) return fail("bad node record");
    m.px[k] = v[0];
    m.py[k] = v[1];
  }
  li += (size_t)m.nEdges;  // edge records
  m.corner.resize(4 * (size_t)m.nElems);
  m.kind.resize(4 * (size_t)m.nElems);
  m.cx.assign(4 * (size_t)m.nElems, {});
  m.cy.assign(4 * (size_t)m.nElems, {});
  m.bc.assign(4 * (size_t)m.nElems, 1);
  for (int e = 0; e < m.nElems; ++e) {
    if (!numbers(li++, v) || v.size() < 4) return fail("bad element node record");
    for (int k = 0; k < 4; ++k) {
      m.corner[4 * e + k] = (int)v[k];
      if (m.corner[4 * e + k] < 1 || m.corner[4 * e + k] > m.nNodes) return fail("element node out of range");
    }
    if (!numbers(li++, v) || v.size() < 4) return fail("bad side-kind record");
    for (int k = 0; k < 4; ++k) m.kind[4 * e + k] = (int)v[k];
    for (int k = 0; k < 4; ++k) {
      if (m.kind[4 * e + k] == 0) continue;
      if (m.kind[4 * e + k] != 1) return fail("side kind other than 0 or 1");
      auto& X = m.cx[4 * e + k];
      auto& Y = m.cy[4 * e + k];
      for (int j = 0; j <= m.gdeg; ++j) {
        if (!numbers(li++, v) || v.size() < 2) return fail("bad curve point");
        X.push_back(v[0]);
        Y.push_back(v[1]);
      }
    }
    if (li >= lines.size()) return fail("missing side names");
    std::istringstream names(lines[li++]);
    for (int k = 0; k < 4; ++k) {
      std::string w;
      if (!(names >> w)) return fail("fewer than 4 side names");
      m.bc[4 * e + k] = ism_flag(w);
    }
  }
  return SELF_OK;
}

// a side curve: interpolant of degree g through points at the Chebyshev-Gauss-Lobatto nodes
struct SideCurve {
  Interp1D I;
  std::vector<double> x, y;
  void at(double s, double& ox, double& oy) const {
    std::vector<double> l(x.size());
    I.basis(s, l.data());
    ox = oy = 0.0;
    for (size_t j = 0; j < x.size(); ++j) ox += l[j] * x[j], oy += l[j] * y[j];
  }
  void slope(double s, double& ox, double& oy) const {
    std::vector<double> l(x.size());
    I.dbasis(s, l.data());
    ox = oy = 0.0;
    for (size_t j = 0; j < x.size(); ++j) ox += l[j] * x[j], oy += l[j] * y[j];
  }
};

// Coons patch of the S, E, N, W curves (S, N parametrised by s; W, E by p) and its covariant metrics
void coons(const SideCurve* c, double s, double p, double* P, double* cov) {
  double sw[2], se[2], nw[2], ne[2], S[2], E[2], Nn[2], W[2], dS[2], dE[2], dN[2], dW[2];
  c[0].at(-1.0, sw[0], sw[1]);
  c[0].at(1.0, se[0], se[1]);
  c[2].at(-1.0, nw[0], nw[1]);
  c[2].at(1.0, ne[0], ne[1]);
  c[0].at(s, S[0], S[1]);
  c[2].at(s, Nn[0], Nn[1]);
  c[3].at(p, W[0], W[1]);
  c[1].at(p, E[0], E[1]);
  c[0].slope(s, dS[0], dS[1]);
  c[2].slope(s, dN[0], dN[1]);
  c[3].slope(p, dW[0], dW[1]);
  c[1].slope(p, dE[0], dE[1]);
  const double am = 0.5 * (1.0 - s), ap = 0.5 * (1.0 + s), bm = 0.5 * (1.0 - p), bp = 0.5 * (1.0 + p);
  for (int d = 0; d < 2; ++d) {
    const double bil = bm * (am * sw[d] + ap * se[d]) + bp * (am * nw[d] + ap * ne[d]);
    P[d] = am * W[d] + ap * E[d] + bm * S[d] + bp * Nn[d] - bil;
    // d/ds and d/dp of the blend
    const double ds = 0.5 * (E[d] - W[d]) + bm * (dS[d] - 0.5 * (se[d] - sw[d])) + bp * (dN[d] - 0.5 * (ne[d] - nw[d]));
    const double dp = 0.5 * (Nn[d] - S[d]) + am * (dW[d] - 0.5 * (nw[d] - sw[d])) + ap * (dE[d] - 0.5 * (ne[d] - se[d]));
    cov[2 * d] = ds;      // dxds, dyds
    cov[2 * d + 1] = dp;  // dxdp, dydp
  }
}

}  // namespace

int self_mesh_ism_counts(const char* path, int* nEl, int* nEdges, int* nNodes, int* geomDegree) {
  if (!path || !nEl || !nEdges || !nNodes) return SELF_ERR_INVALID;
  IsmMesh m;
  int rc = ism_read(path, m, true);
  if (rc) return rc;
  *nEl = m.nElems;
  *nEdges = m.nEdges;
  *nNodes = m.nNodes;
  if (geomDegree) *geomDegree = m.gdeg;
  return SELF_OK;
}

int self_mesh_ism_build(const char* path, int N, int quad, int* edges, int* elemNodes, int* nodeType, int* n2e_ptr,
                        int* n2e_elem, int* n2e_local, double* X, double* Y, double* dxds, double* dxdp,
                        double* dyds, double* dydp, double* J, double* nhx, double* nhy, double* nlen, double* bx,
                        double* by) {
  if (!path) return SELF_ERR_INVALID;
  if (N < 1 || N > 15) return set_error(nullptr, SELF_ERR_INVALID, "polynomial degree %d outside 1..15", N);
  IsmMesh m;
  int rc = ism_read(path, m, false);
  if (rc) return rc;
  const int n = N + 1, nEl = m.nElems;
  std::vector<double> xq, wq;
  quadrature(N, quad, xq, wq);
  std::vector<double> cgl(m.gdeg + 1);
  for (int j = 0; j <= m.gdeg; ++j) cgl[j] = -std::cos(j * (kPi / m.gdeg));
  static const int corner_of[4][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}};  // S, E, N, W: first and last corner
  for (int k = 0; k < m.nNodes; ++k) nodeType[k] = 0;
  for (int e = 0; e < nEl; ++e) {
    for (int k = 0; k < 4; ++k) elemNodes[4 * e + k] = m.corner[4 * e + k];
    SideCurve c[4];
    for (int side = 0; side < 4; ++side) {
      c[side].I.build(cgl);
      if (m.kind[4 * e + side] == 0) {
        const int a = m.corner[4 * e + corner_of[side][0]] - 1, b = m.corner[4 * e + corner_of[side][1]] - 1;
        c[side].x.resize(m.gdeg + 1);
        c[side].y.resize(m.gdeg + 1);
        for (int j = 0; j <= m.gdeg; ++j) {
          const double t = 0.5 * (cgl[j] + 1.0);
          c[side].x[j] = m.px[a] + (m.px[b] - m.px[a]) * t;
          c[side].y[j] = m.py[a] + (m.py[b] - m.py[a]) * t;
        }
      } else {
        c[side].x = m.cx[4 * e + side];
        c[side].y = m.cy[4 * e + side];
      }
    }
    const size_t o = (size_t)n * n * e;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double P[2], cov[4];
        coons(c, xq[i], xq[j], P, cov);
        const size_t id = o + i + (size_t)n * j;
        X[id] = P[0];
        Y[id] = P[1];
        dxds[id] = cov[0];
        dxdp[id] = cov[1];
        dyds[id] = cov[2];
        dydp[id] = cov[3];
        J[id] = cov[0] * cov[3] - cov[1] * cov[2];
      }
    for (int side = 0; side < 4; ++side)
      for (int k = 0; k < n; ++k) {
        const double s = (side == 1) ? 1.0 : (side == 3) ? -1.0 : xq[k];
        const double p = (side == 0) ? -1.0 : (side == 2) ? 1.0 : xq[k];
        double P[2], cov[4];
        coons(c, s, p, P, cov);
        const double Jb = cov[0] * cov[3] - cov[1] * cov[2];
        const double sg = Jb > 0 ? 1.0 : -1.0;
        double d0, d1;  // outward normal scaled by the side's length element
        switch (side) {
          case 0: d0 = sg * cov[2]; d1 = -sg * cov[0]; break;
          case 2: d0 = -sg * cov[2]; d1 = sg * cov[0]; break;
          case 3: d0 = -sg * cov[3]; d1 = sg * cov[1]; break;
          default: d0 = sg * cov[3]; d1 = -sg * cov[1]; break;
        }
        const size_t ib = (size_t)k + n * (side + 4 * (size_t)e);
        const double len = std::sqrt(d0 * d0 + d1 * d1);
        nhx[ib] = d0 / len;
        nhy[ib] = d1 / len;
        nlen[ib] = len;
        bx[ib] = P[0];
        by[ib] = P[1];
      }
  }
  // edges in order of first appearance; keyed by the corner-node pair
  std::unordered_map<unsigned long long, int> seen;
  seen.reserve(2 * (size_t)m.nEdges);
  std::vector<int> first_node, last_node;
  int ne = 0;
  for (int e = 0; e < nEl; ++e)
    for (int side = 0; side < 4; ++side) {
      const int a = m.corner[4 * e + corner_of[side][0]], b = m.corner[4 * e + corner_of[side][1]];
      const unsigned long long key = ((unsigned long long)std::min(a, b) << 32) | (unsigned)std::max(a, b);
      auto it = seen.find(key);
      if (it == seen.end()) {
        if (ne >= m.nEdges) return set_error(nullptr, SELF_ERR_INVALID, "%s: more sides than edges", path);
        seen.emplace(key, ne);
        int* E = edges + 6 * ne;
        E[0] = e + 1;
        E[1] = side + 1;
        E[2] = SELF_NO_NORMAL_FLOW;  // default boundary kind until a second element claims the edge
        E[3] = 0;
        first_node.push_back(a);
        last_node.push_back(b);
        ++ne;
      } else {
        int* E = edges + 6 * it->second;
        E[2] = e + 1;
        E[3] = (a == first_node[it->second]) ? side + 1 : -(side + 1);
      }
    }
  if (ne != m.nEdges) return set_error(nullptr, SELF_ERR_INVALID, "%s: %d edges built, %d in the file", path, ne, m.nEdges);
  for (int k = 0; k < ne; ++k) {
    int* E = edges + 6 * k;
    const int fl = m.bc[4 * (E[0] - 1) + E[1] - 1];
    if (fl < 0) {  // a named boundary condition on the primary side
      E[2] = fl;
      nodeType[first_node[k] - 1] = fl;
      nodeType[last_node[k] - 1] = fl;
    }
    E[4] = (E[3] < 0) ? N - 1 : 1;
    E[5] = (E[3] < 0) ? -1 : 1;
  }
  std::vector<int> cnt(m.nNodes + 1, 0);
  for (int e = 0; e < nEl; ++e)
    for (int c = 0; c < 4; ++c) cnt[elemNodes[4 * e + c]]++;
  n2e_ptr[0] = 0;
  for (int i = 0; i < m.nNodes; ++i) n2e_ptr[i + 1] = n2e_ptr[i] + cnt[i + 1];
  std::vector<int> pos(n2e_ptr, n2e_ptr + m.nNodes);
  for (int e = 0; e < nEl; ++e)
    for (int c = 0; c < 4; ++c) {
      const int nd = elemNodes[4 * e + c] - 1;
      n2e_elem[pos[nd]] = e + 1;
      n2e_local[pos[nd]] = c + 1;
      pos[nd]++;
    }
  return SELF_OK;
}

// CalculateBathymetryGradient: the DG weak derivative of h with the element's own boundary values.
int self_sw_bathymetry_gradient(int N, int nEl, const double* dS, const double* dP, const double* qw,
                                const double* lW, const double* lE, const double* lS, const double* lN,
                                const double* dxds, const double* dxdp, const double* dyds, const double* dydp,
                                const double* J, const double* nhx, const double* nhy, const double* nlen,
                                const double* h, double* dhdx, double* dhdy) {
  if (N < 1 || N > 15 || nEl < 1) return set_error(nullptr, SELF_ERR_INVALID, "bad sizes");
  const int n = N + 1;
  std::vector<double> hb(4 * n), f(2 * n), out(2 * n * n);
  for (int e = 0; e < nEl; ++e) {
    const size_t o = (size_t)n * n * e;
    const double* he = h + o;
    for (int k = 0; k < n; ++k) {
      double s = 0, no = 0, w = 0, ea = 0;
      for (int m = 0; m < n; ++m) {
        s += lS[m] * he[k + n * m];
        no += lN[m] * he[k + n * m];
        w += lW[m] * he[m + n * k];
        ea += lE[m] * he[m + n * k];
      }
      hb[k + n * 0] = s;
      hb[k + n * 1] = ea;
      hb[k + n * 2] = no;
      hb[k + n * 3] = w;
    }
    auto nrm = [&](int side, int k, int c) {
      size_t ib = (size_t)k + n * (side + 4 * (size_t)e);
      return (c == 0 ? nhx[ib] : nhy[ib]) * nlen[ib];
    };
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < n; ++i) {
        f[i] = dydp[o + i + n * j] * he[i + n * j];
        f[i + n] = -dxdp[o + i + n * j] * he[i + n * j];
      }
      for (int c = 0; c < 2; ++c) {
        double fR = hb[j + n * 1] * nrm(1, j, c), fL = hb[j + n * 3] * nrm(3, j, c);
        for (int i = 0; i < n; ++i) {
          double a = 0;
          for (int m = 0; m < n; ++m) a += dS[i + m * n] * f[m + c * n];
          out[i + n * j + c * n * n] = a + (fR * lE[i] + fL * lW[i]) / qw[i];
        }
      }
    }
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) {
        f[j] = -dyds[o + i + n * j] * he[i + n * j];
        f[j + n] = dxds[o + i + n * j] * he[i + n * j];
      }
      for (int c = 0; c < 2; ++c) {
        double fR = hb[i + n * 2] * nrm(2, i, c), fL = hb[i + n * 0] * nrm(0, i, c);
        for (int j = 0; j < n; ++j) {
          double a = 0;
          for (int m = 0; m < n; ++m) a += dP[j + m * n] * f[m + c * n];
          a += (fR * lN[j] + fL * lS[j]) / qw[j];
          out[i + n * j + c * n * n] = (out[i + n * j + c * n * n] + a) / J[o + i + n * j];
        }
      }
    }
    for (int k = 0; k < n * n; ++k) {
      dhdx[o + k] = out[k];
      dhdy[o + k] = out[k + n * n];
    }
  }
  return SELF_OK;
}

// ------------------------------------------------------------------------------------------------ pickup files
// Direct-access, big-endian, unformatted records of (N+1)^2 doubles (i fastest) without record markers, as the
// reference writes them (WritePickup_ShallowWater / ReadPickup_ShallowWater, ConservativeShallowWaterClass.f90:
// 2013-2130; WritePickup_Advection / ReadPickup_Advection, AdvectionClass.f90:2040-2171): for every element, for
// every field in order, recs[f] records taken from fields[f] at element offset (e * recs[f] + r) * (N+1)^2.
namespace {
inline uint64_t swap64(uint64_t v) {
  uint64_t r = 0;
  for (int b = 0; b < 8; ++b) r |= ((v >> (8 * b)) & 0xffULL) << (8 * (7 - b));
  return r;
}
int pickup_args(int N, int nEl, int nfields, const void* fields, const int* recs) {
  if (N < 1 || nEl < 1 || nfields < 1 || !fields || !recs) return SELF_ERR_INVALID;
  for (int f = 0; f < nfields; ++f)
    if (recs[f] < 1) return SELF_ERR_INVALID;
  return SELF_OK;
}
}  // namespace

int self_pickup_write(const char* path, int N, int nEl, int nfields, const double* const* fields, const int* recs) {
  if (!path || pickup_args(N, nEl, nfields, fields, recs)) return set_error(nullptr, SELF_ERR_INVALID, "pickup arguments");
  for (int f = 0; f < nfields; ++f)
    if (!fields[f]) return set_error(nullptr, SELF_ERR_INVALID, "pickup field %d is null", f);
  FILE* fp = fopen(path, "wb");
  if (!fp) return set_error(nullptr, SELF_ERR_INVALID, "cannot open %s for writing", path);
  const size_t nn = (size_t)(N + 1) * (N + 1);
  std::vector<uint64_t> rec(nn);
  for (int e = 0; e < nEl; ++e)
    for (int f = 0; f < nfields; ++f)
      for (int r = 0; r < recs[f]; ++r) {
        const double* src = fields[f] + ((size_t)e * recs[f] + r) * nn;
        for (size_t k = 0; k < nn; ++k) {
          uint64_t v;
          std::memcpy(&v, &src[k], 8);
          rec[k] = swap64(v);
        }
        if (fwrite(rec.data(), 8, nn, fp) != nn) {
          fclose(fp);
          return set_error(nullptr, SELF_ERR_INVALID, "short write to %s", path);
        }
      }
  if (fclose(fp) != 0) return set_error(nullptr, SELF_ERR_INVALID, "closing %s failed", path);
  return SELF_OK;
}

int self_pickup_read(const char* path, int N, int nEl, int nfields, double* const* fields, const int* recs) {
  if (!path || pickup_args(N, nEl, nfields, fields, recs)) return set_error(nullptr, SELF_ERR_INVALID, "pickup arguments");
  FILE* fp = fopen(path, "rb");
  if (!fp) return set_error(nullptr, SELF_ERR_INVALID, "cannot open %s", path);
  const size_t nn = (size_t)(N + 1) * (N + 1);
  std::vector<uint64_t> rec(nn);
  for (int e = 0; e < nEl; ++e)
    for (int f = 0; f < nfields; ++f)
      for (int r = 0; r < recs[f]; ++r) {
        if (fread(rec.data(), 8, nn, fp) != nn) {
          fclose(fp);
          return set_error(nullptr, SELF_ERR_INVALID, "%s ends before element %d, field %d", path, e + 1, f);
        }
        if (!fields[f]) continue;  // a field the caller does not want
        double* dst = fields[f] + ((size_t)e * recs[f] + r) * nn;
        for (size_t k = 0; k < nn; ++k) {
          const uint64_t v = swap64(rec[k]);
          std::memcpy(&dst[k], &v, 8);
        }
      }
  fclose(fp);
  return SELF_OK;
}

}  // extern "C"
