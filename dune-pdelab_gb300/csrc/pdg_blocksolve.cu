// pdg_blocksolve.cu -- the matrix-free block preconditioners beyond plain
// block Jacobi:
//
//  * iterative block Jacobi (IterativeBlockJacobiPreconditionerLocalOperator,
//    backend/istl/matrixfree/iterativeblockjacobipreconditioner.hh:262-452):
//    every diagonal block system D_e b = d_e is solved by a local BiCGStab
//    (dune-istl BiCGSTABSolver semantics, as the reference instantiates it in
//    test/matrixfree/matrix_free_linear.cc:200-205) preconditioned by the
//    weighted inverse point diagonal of D_e (LocalPointJacobiPreconditioner,
//    :28-80), to BlockSolverOptions' reduction / iteration cap (:202-233).
//    On the GPU all local solves run batched in one kernel: one warp-multiple
//    thread group per cell, the local vectors in registers, D_e read from a
//    per-cell block store, reductions by warp shuffles (deterministic order);
//    cells iterate independently and a block retires when its group has
//    converged.
//
//  * block SOR (BlockSORPreconditionerLocalOperator,
//    backend/istl/matrixfree/blocksorpreconditioner.hh:37-296): one forward
//    sweep over the cells in grid order from v = 0,
//        v_e = omega D_e^{-1} (d_e - sum_{f < e} A_ef v_f),
//    with D_e^{-1} applied by any of the block solvers.  Cell e depends only
//    on its lower face neighbours, so the cells of one hyperplane
//    ix+iy+iz = s are independent: the sweep runs hyperplane by hyperplane
//    (nx+ny+nz-2 steps), giving the sequential sweep's result up to rounding.
//    Within step s every cell at or above the hyperplane still holds v = 0,
//    so d_e - sum_{f<e} A_ef v_f = d_e - (J v)_e and the full operator
//    kernel (convection included) restricted to the hyperplane's cells
//    computes it.  The transposed preconditioner (adjoint solves) is the
//    backward sweep with J^T and D_e^{-T}.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pdg_internal.cuh"
#include "pdg_vec.cuh"

namespace pdg {

// ---------------------------------------------------------------------------
// iterative block Jacobi
// ---------------------------------------------------------------------------

// blk[e][j*nb+i] = D[e][i][j] (column-major) and invdiag[e][i] = 1 / D_ii
template <typename T>
__global__ void k_bj_pack(long ncell, int nb, const double *__restrict__ D, T *__restrict__ blk,
                          T *__restrict__ invdiag) {
  const long n = ncell * nb * nb;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / ((long)nb * nb);
    const int r = (int)(t - e * nb * nb);
    const int i = r / nb, j = r - (r / nb) * nb;
    const double v = D[t];
    blk[e * nb * nb + (long)j * nb + i] = (T)v;
    if (i == j) invdiag[e * nb + i] = (T)(1.0 / v);
  }
}

// sum over the thread group of one cell (G = 32 * wpc threads); wpc > 1
// goes through shared memory, every thread of the block takes part
template <int WPC>
__device__ __forceinline__ double group_sum(double v, double *scratch, int cs, int warp_in_cell,
                                            int lane) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (WPC == 1) return v;
  __syncthreads();
  if (lane == 0) scratch[cs * WPC + warp_in_cell] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int w = 0; w < WPC; w++) s += scratch[cs * WPC + w];
  return s;
}

// Batched local BiCGStab on D_e b = d_e for the listed cells; v_e = scale * b.
template <typename T, int WPC>
__global__ void __launch_bounds__(256)
    k_bj_iter(long ncell, int nb, const T *__restrict__ blk, const T *__restrict__ invdiag,
              const T *__restrict__ d, T *__restrict__ v, int transpose,
              const int *__restrict__ skip, const int *__restrict__ cells, int ncells, T scale,
              double red, int maxit, int precond, double weight, int *__restrict__ iters) {
  constexpr int G = 32 * WPC;
  if (skip && *skip) return;
  const int CPB = blockDim.x / G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *scratch = reinterpret_cast<double *>(smem_raw);        // [CPB][WPC]
  T *yb = reinterpret_cast<T *>(scratch + CPB * WPC);            // [CPB][nb]
  const int t = threadIdx.x, cs = t / G, l = t - cs * G, lane = t & 31, wic = l >> 5;
  const long li = (long)blockIdx.x * CPB + cs;
  const bool active = cells ? li < ncells : li < ncell;
  const long e = cells ? (active ? (long)cells[li] : 0) : li;
  const bool own = active && l < nb;
  T *ys = yb + cs * nb;
  const T *B = blk + (active ? e : 0) * (long)nb * nb;
  const T idg = own ? (T)(precond ? weight * (double)invdiag[e * nb + l] : 1.0) : T(0);

  auto matvec = [&](T in) -> T {
    __syncthreads();
    if (own) ys[l] = in;
    __syncthreads();
    T s = T(0);
    if (own) {
      if (!transpose)
        for (int j = 0; j < nb; j++) s += B[(long)j * nb + l] * ys[j];
      else
        for (int j = 0; j < nb; j++) s += B[(long)l * nb + j] * ys[j];
    }
    return s;
  };
  auto gsum = [&](double val) -> double { return group_sum<WPC>(val, scratch, cs, wic, lane); };

  T x = T(0), r = own ? d[e * nb + l] : T(0);
  const T rt = r;
  T p = T(0), vv = T(0);
  double def0 = sqrt(gsum((double)r * r));
  bool done = !(def0 >= 1e-30) || !active;   // converged at 0 (or NaN / inactive)
  double it_done = 0.0;
  double rho = 1.0, alpha = 1.0, omega = 1.0;
  const double EPS = 1e-80;
  for (double it = 0.5; it < maxit; it += 0.5) {
    if (!__syncthreads_or(!done)) break;
    const double rho_new = gsum((double)rt * r);
    bool brk = fabs(rho) <= EPS || fabs(omega) <= EPS;
    if (!done && brk) { done = true; it_done = it; }
    if (!done) {
      if (it < 1.0) p = r;
      else {
        const double beta = (rho_new / rho) * (alpha / omega);
        p = (T)(beta * ((double)p - omega * (double)vv) + (double)r);
      }
    }
    T y = idg * p;
    vv = matvec(y);
    const double h = gsum((double)rt * vv);
    if (!done && fabs(h) < EPS) { done = true; it_done = it; }
    if (!done) {
      alpha = rho_new / h;
      x = (T)((double)x + alpha * (double)y);
      r = (T)((double)r - alpha * (double)vv);
    }
    double nrm = sqrt(gsum((double)r * r));
    if (!done && (!(nrm < INFINITY) || nrm < def0 * red || nrm < 1e-30)) {
      done = true;
      it_done = it;
    }
    const double it2 = it + 0.5;
    y = idg * r;
    const T tv = matvec(y);
    const double tr = gsum((double)tv * r);
    const double tt = gsum((double)tv * tv);
    if (!done) {
      omega = tr / tt;
      x = (T)((double)x + omega * (double)y);
      r = (T)((double)r - omega * (double)tv);
      rho = rho_new;
    }
    nrm = sqrt(gsum((double)r * r));
    if (!done && (!(nrm < INFINITY) || nrm < def0 * red || nrm < 1e-30)) {
      done = true;
      it_done = it2;
    }
    it = it2;
    if (!done && it + 0.5 >= maxit) it_done = maxit;
  }
  if (own) v[e * nb + l] = scale * x;
  if (active && l == 0 && iters) iters[e] = (int)ceil(it_done);
}

int bj_iterative_setup(pdg_context *ctx, int precision) {
  double *D = nullptr;
  PDG_TRY(diag_blocks(ctx, &D));
  PrecData &pd = ctx->prec[precision];
  const int nb = ctx->nb;
  const size_t es = precision == PDG_F64 ? sizeof(double) : sizeof(float);
  const size_t nblk = (size_t)ctx->ncell * nb * nb;
  if (cudaMalloc(&pd.blk, nblk * es) != cudaSuccess ||
      cudaMalloc(&pd.invdiag, (size_t)ctx->ndof * es) != cudaSuccess ||
      cudaMalloc(&pd.iters, sizeof(int) * ctx->ncell) != cudaSuccess) {
    cudaFree(D);
    return set_error(PDG_ECUDA, "out of device memory for the block store");
  }
  long g = ((long)nblk + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  if (precision == PDG_F64)
    k_bj_pack<double><<<(unsigned)g, 256, 0, ctx->stream>>>(ctx->ncell, nb, D, (double *)pd.blk,
                                                            (double *)pd.invdiag);
  else
    k_bj_pack<float><<<(unsigned)g, 256, 0, ctx->stream>>>(ctx->ncell, nb, D, (float *)pd.blk,
                                                           (float *)pd.invdiag);
  PDG_CUDA_TRY(cudaMemsetAsync(pd.iters, 0, sizeof(int) * ctx->ncell, ctx->stream));
  PDG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  cudaFree(D);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <typename T, int WPC>
static int bj_iter_launch(pdg_context *ctx, const PrecData &pd, const T *d, T *v, int transpose,
                          const int *skip, const int *cells, int ncells, T scale) {
  const int G = 32 * WPC;
  const int CPB = std::max(1, 256 / G);
  const long work = cells ? ncells : ctx->ncell;
  const unsigned blocks = (unsigned)((work + CPB - 1) / CPB);
  const size_t smem = sizeof(double) * CPB * WPC + sizeof(T) * CPB * ctx->nb;
  const pdg_prec_options &o = ctx->popt;
  k_bj_iter<T, WPC><<<blocks, CPB * G, smem, ctx->stream>>>(
      ctx->ncell, ctx->nb, (const T *)pd.blk, (const T *)pd.invdiag, d, v, transpose, skip, cells,
      ncells, scale, o.block_reduction, o.block_maxit, o.block_precondition, o.block_weight,
      pd.iters);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

template <typename T>
int bj_iterative_apply(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip,
                       const int *cells, int ncells, T scale) {
  const PrecData &pd = ctx->prec[std::is_same<T, double>::value ? PDG_F64 : PDG_F32];
  if (!pd.blk) return set_error(PDG_ESTATE, "iterative block Jacobi not set up");
  if ((cells ? ncells : ctx->ncell) <= 0) return PDG_OK;
  const int wpc = (ctx->nb + 31) / 32;
  switch (wpc) {
    case 1: return bj_iter_launch<T, 1>(ctx, pd, d, v, transpose, skip, cells, ncells, scale);
    case 2: return bj_iter_launch<T, 2>(ctx, pd, d, v, transpose, skip, cells, ncells, scale);
    case 3:
    case 4: return bj_iter_launch<T, 4>(ctx, pd, d, v, transpose, skip, cells, ncells, scale);
    default: return set_error(PDG_EUNSUPPORTED, "block size not supported");
  }
}

template int bj_iterative_apply<double>(pdg_context *, const double *, double *, int, const int *,
                                        const int *, int, double);
template int bj_iterative_apply<float>(pdg_context *, const float *, float *, int, const int *,
                                       const int *, int, float);

// ---------------------------------------------------------------------------
// block SOR
// ---------------------------------------------------------------------------

int sor_setup(pdg_context *ctx) {
  if (ctx->basis == PDG_BASIS_LEGENDRE)
    return set_error(PDG_EUNSUPPORTED, "block SOR needs a nodal basis");
  if (ctx->hp_cells) return PDG_OK;
  const int d = ctx->dim;
  const long nx = ctx->cfg.cells[0], ny = ctx->cfg.cells[1];
  const long nz = d == 3 ? ctx->cfg.cells[2] : 1;
  const int nh = (int)(nx + ny + nz - 2);
  std::vector<long> count(nh + 1, 0);
  for (long e = 0; e < ctx->ncell; e++) {
    const long s = e % nx + (e / nx) % ny + e / (nx * ny);
    count[s]++;
  }
  long *off = new long[nh + 2];
  off[0] = 0;
  for (int s = 0; s <= nh; s++) off[s + 1] = off[s] + count[s];
  std::vector<int> cells(ctx->ncell);
  std::vector<long> pos(off, off + nh + 1);
  for (long e = 0; e < ctx->ncell; e++) {
    const long s = e % nx + (e / nx) % ny + e / (nx * ny);
    cells[pos[s]++] = (int)e;
  }
  int *dev = nullptr;
  if (cudaMalloc(&dev, sizeof(int) * ctx->ncell) != cudaSuccess) {
    delete[] off;
    return set_error(PDG_ECUDA, "out of device memory for the sweep order");
  }
  if (cudaMemcpy(dev, cells.data(), sizeof(int) * ctx->ncell, cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    cudaFree(dev);
    delete[] off;
    return set_error(PDG_ECUDA, "copy of the sweep order failed");
  }
  ctx->hp_cells = dev;
  ctx->hp_off = off;
  ctx->hp_n = nh + 1;
  return PDG_OK;
}

void sor_free(pdg_context *ctx) {
  if (ctx->hp_cells) cudaFree(ctx->hp_cells);
  delete[] ctx->hp_off;
  void *bufs[] = {ctx->sor_a64, ctx->sor_d64, ctx->sor_v64,
                  ctx->sor_a32, ctx->sor_d32, ctx->sor_v32};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (int i = 0; i < 8; i++) {
    cudaGraphExec_t &g = (&ctx->sor_graph[0][0][0])[i];
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  ctx->hp_cells = nullptr;
  ctx->hp_off = nullptr;
  ctx->sor_a64 = ctx->sor_d64 = ctx->sor_v64 = nullptr;
  ctx->sor_a32 = ctx->sor_d32 = ctx->sor_v32 = nullptr;
  ctx->hp_n = 0;
}

// the sweep body on the given buffers: v = 0, then per hyperplane
// a = d - (J v) on its cells and v = omega D^{-1} a there
template <typename T>
static int sor_sweep(pdg_context *ctx, const T *d, T *v, T *a, int transpose, const int *skip) {
  const bool dbl = std::is_same<T, double>::value;
  const T *K = dbl ? (const T *)ctx->K64 : (const T *)ctx->K32;
  const T *c = dbl ? (const T *)ctx->c64 : (const T *)ctx->c32;
  const T *tab = dbl ? (const T *)ctx->tab64 : (const T *)ctx->tab32;
  const T omega = (T)ctx->popt.omega;
  PDG_TRY(vec_fill<T>(ctx, ctx->ndof, v, T(0)));
  for (int q = 0; q < ctx->hp_n; q++) {
    const int s = transpose ? ctx->hp_n - 1 - q : q;
    const long b = ctx->hp_off[s], cnt = ctx->hp_off[s + 1] - b;
    if (cnt == 0) continue;
    const int *cl = ctx->hp_cells + b;
    // a_e = d_e - (J v)_e on the hyperplane (lower neighbours hold new values)
    ApplyArgs<T> aa{v, a, d, T(-1), 0, transpose, 0, skip, cl, (int)cnt};
    PDG_TRY(launch_apply<T>(ctx, aa, K, c, tab));
    // v_e = omega D_e^{-1} a_e
    PDG_TRY(block_solve<T>(ctx, a, v, transpose, skip, cl, (int)cnt, omega));
  }
  return PDG_OK;
}

// The 2(nx+ny+nz-2) launches of a sweep are latency bound, so the sweep is
// captured once per operator / preconditioner generation as a CUDA graph on
// fixed input/output buffers and replayed: d is copied in, v copied out.
// The first sweep of a generation runs eagerly (it builds any lazily
// created per-cell records outside the capture).
template <typename T>
int sor_apply(pdg_context *ctx, const T *d, T *v, int transpose, const int *skip) {
  PDG_TRY(sor_setup(ctx));
  const int pi = std::is_same<T, double>::value ? 0 : 1;
  T *&a = *reinterpret_cast<T **>(pi == 0 ? (void *)&ctx->sor_a64 : (void *)&ctx->sor_a32);
  T *&D = *reinterpret_cast<T **>(pi == 0 ? (void *)&ctx->sor_d64 : (void *)&ctx->sor_d32);
  T *&V = *reinterpret_cast<T **>(pi == 0 ? (void *)&ctx->sor_v64 : (void *)&ctx->sor_v32);
  for (T **b : {&a, &D, &V})
    if (!*b) PDG_CUDA_TRY(cudaMalloc(b, sizeof(T) * ctx->ndof));
  const int tr = transpose ? 1 : 0, sk = skip ? 1 : 0;
  cudaGraphExec_t &g = ctx->sor_graph[pi][tr][sk];
  unsigned &gen = ctx->sor_graph_gen[pi][tr][sk];
  if (!g || gen != ctx->op_gen) {
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
    // eager sweep (also the result of this call)
    PDG_TRY(sor_sweep<T>(ctx, d, v, a, transpose, skip));
    cudaGraph_t graph = nullptr;
    PDG_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int st = sor_sweep<T>(ctx, D, V, a, transpose, skip);
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (st != PDG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    PDG_CUDA_TRY(ce);
    const cudaError_t ie = cudaGraphInstantiate(&g, graph, 0);
    cudaGraphDestroy(graph);
    PDG_CUDA_TRY(ie);
    gen = ctx->op_gen;
    return PDG_OK;
  }
  PDG_CUDA_TRY(cudaMemcpyAsync(D, d, sizeof(T) * ctx->ndof, cudaMemcpyDeviceToDevice, ctx->stream));
  PDG_CUDA_TRY(cudaGraphLaunch(g, ctx->stream));
  PDG_CUDA_TRY(cudaMemcpyAsync(v, V, sizeof(T) * ctx->ndof, cudaMemcpyDeviceToDevice, ctx->stream));
  return PDG_OK;
}

template int sor_apply<double>(pdg_context *, const double *, double *, int, const int *);
template int sor_apply<float>(pdg_context *, const float *, float *, int, const int *);

}  // namespace pdg
