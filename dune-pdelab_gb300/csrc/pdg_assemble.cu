// pdg_assemble.cu -- the assembled Jacobian of the operator on the GPU
// (GridOperator::jacobian, gridoperator/gridoperator.hh:184-189, driving
// ConvectionDiffusionDG::jacobian_volume / _skeleton / _boundary,
// localoperator/convectiondiffusiondg.hh:198-266, 483-669, 901-1044), its
// block-sparse product, and its export in ISTL's BCRS layout.
//
// Assembly by probing the matrix-free operator: with cells coloured by
// (ix mod 3, iy mod 3, iz mod 3), no cell is face-adjacent or equal to two
// cells of one colour, so J applied to the unit vector of local basis
// function j on every cell of colour c yields, in every cell e, column j of
// the block (e, e') for the one cell e' of colour c in e's closed face
// neighbourhood.  3^d * n applies assemble every block exactly as the apply
// computes it (convection and boundary terms included).
//
// Storage: fixed slots per cell, [ncell][2d+1][n][n], slot 0 the diagonal
// block and slot 1+f the coupling through face f (-x,+x,-y,+y,-z,+z); each
// block column-major (entry (i,j) at j*n + i) so that the block product
// reads consecutive addresses across threads.  Missing neighbours leave zero
// blocks.  The export converts to compressed rows with ascending column
// blocks and row-major blocks (BCRSMatrix<FieldMatrix<double,n,n>>).
#include <vector>

#include "pdg_internal.cuh"
#include "pdg_vec.cuh"

namespace pdg {

struct Grid3 {
  int nc[3];
  int dim;
};

__device__ __forceinline__ void cell_ijk(const Grid3 &g, long e, int *ix) {
  ix[0] = (int)(e % g.nc[0]);
  const long r = e / g.nc[0];
  ix[1] = (int)(r % g.nc[1]);
  ix[2] = (int)(r / g.nc[1]);
}

// neighbour across face f, or -1
__device__ __forceinline__ long face_neighbour(const Grid3 &g, long e, const int *ix, int f) {
  const int dir = f >> 1;
  const long stride = dir == 0 ? 1 : (dir == 1 ? (long)g.nc[0] : (long)g.nc[0] * g.nc[1]);
  if (f & 1) return ix[dir] + 1 < g.nc[dir] ? e + stride : -1;
  return ix[dir] > 0 ? e - stride : -1;
}

__device__ __forceinline__ int colour_of(const Grid3 &g, const int *ix) {
  int c = 0;
  for (int j = g.dim - 1; j >= 0; j--) c = c * 3 + ix[j] % 3;
  return c;
}

// x = sum over cells of colour c of the unit vector of local index j
__global__ void k_probe_fill(Grid3 g, long ncell, int nb, int c, int j, double *x) {
  const long n = ncell * nb;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / nb;
    const int i = (int)(t - e * nb);
    int ix[3];
    cell_ijk(g, e, ix);
    x[t] = (i == j && colour_of(g, ix) == c) ? 1.0 : 0.0;
  }
}

// column j of block (e, slot) = y_e for the slot whose cell has colour c
__global__ void k_probe_scatter(Grid3 g, long ncell, int nb, int c, int j, const double *y,
                                double *A) {
  const int ns = 2 * g.dim + 1;
  const long n = ncell * nb;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / nb;
    const int i = (int)(t - e * nb);
    int ix[3];
    cell_ijk(g, e, ix);
    for (int s = 0; s < ns; s++) {
      long nbc = e;
      int jx[3] = {ix[0], ix[1], ix[2]};
      if (s > 0) {
        const int f = s - 1;
        nbc = face_neighbour(g, e, ix, f);
        if (nbc < 0) continue;
        jx[f >> 1] += (f & 1) ? 1 : -1;
      }
      if (colour_of(g, jx) != c) continue;
      A[((e * ns + s) * nb + j) * (long)nb + i] = y[t];
      break;
    }
  }
}

// y = alpha * A x (+ y if accumulate) (+ add); A^T with `transpose`.
// One thread per row entry; the block product walks the 2d+1 slots.
__global__ void k_bcrs_apply(Grid3 g, long ncell, int nb, const double *__restrict__ A,
                             const double *__restrict__ x, double *__restrict__ y,
                             const double *__restrict__ add, double alpha, int accumulate,
                             int transpose, const int *skip) {
  if (skip && *skip) return;
  const int ns = 2 * g.dim + 1;
  const long n = ncell * nb;
  const long bs = (long)nb * nb;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / nb;
    const int i = (int)(t - e * nb);
    int ix[3];
    cell_ijk(g, e, ix);
    double s = 0.0;
    for (int sl = 0; sl < ns; sl++) {
      long nbc = e;
      int msl = 0;   // slot of e in the neighbour's row (transpose)
      if (sl > 0) {
        const int f = sl - 1;
        nbc = face_neighbour(g, e, ix, f);
        if (nbc < 0) continue;
        msl = 1 + (f ^ 1);
      }
      const double *xb = x + nbc * nb;
      if (!transpose) {
        // row i of A_(e,nbc): entries (i, j) at j*nb + i
        const double *B = A + (e * ns + sl) * bs;
        for (int j = 0; j < nb; j++) s += B[(long)j * nb + i] * xb[j];
      } else {
        // row i of (A_(nbc,e))^T = column i of A_(nbc,e): contiguous
        const double *B = A + (nbc * ns + msl) * bs + (long)i * nb;
        for (int j = 0; j < nb; j++) s += B[j] * xb[j];
      }
    }
    double r = alpha * s;
    if (accumulate) r += y[t];
    if (add) r += add[t];
    y[t] = r;
  }
}

// compressed export: values[(rowptr[e] + k) * n*n + i*n + j] = A(e, col_k)(i, j)
__global__ void k_bcrs_export(Grid3 g, long ncell, int nb, const double *__restrict__ A,
                              const long *__restrict__ rowptr, double *__restrict__ out) {
  const int ns = 2 * g.dim + 1;
  const long bs = (long)nb * nb;
  const long n = ncell * bs;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / bs;
    const int r = (int)(t - e * bs);
    const int i = r / nb, j = r - (r / nb) * nb;
    int ix[3];
    cell_ijk(g, e, ix);
    // ascending column order: -z, -y, -x, self, +x, +y, +z
    int k = 0;
    for (int q = 0; q < ns; q++) {
      int sl;
      if (q < g.dim) sl = 1 + 2 * (g.dim - 1 - q);        // lower faces, far first
      else if (q == g.dim) sl = 0;
      else sl = 1 + 2 * (q - g.dim - 1) + 1;              // upper faces, near first
      if (sl > 0 && face_neighbour(g, e, ix, sl - 1) < 0) continue;
      out[(rowptr[e] + k) * bs + (long)i * nb + j] = A[(e * ns + sl) * bs + (long)j * nb + i];
      k++;
    }
  }
}

static Grid3 grid_of(const pdg_context *ctx) {
  Grid3 g;
  g.dim = ctx->dim;
  for (int j = 0; j < 3; j++) g.nc[j] = j < ctx->dim ? ctx->cfg.cells[j] : 1;
  return g;
}

static unsigned grid_for(long n) {
  long b = (n + 255) / 256;
  if (b > 152L * 32) b = 152L * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

long jacobian_nnz_blocks(const pdg_context *ctx) {
  long nnz = ctx->ncell;
  for (int dir = 0; dir < ctx->dim; dir++) {
    long faces = 1;
    for (int j = 0; j < ctx->dim; j++) faces *= j == dir ? ctx->cfg.cells[j] - 1 : ctx->cfg.cells[j];
    nnz += 2 * faces;
  }
  return nnz;
}

int jacobian_rowptr(const pdg_context *ctx, long *rowptr, long *colind) {
  const int d = ctx->dim;
  const long nx = ctx->cfg.cells[0], ny = ctx->cfg.cells[1];
  const long nz = d == 3 ? ctx->cfg.cells[2] : 1;
  long k = 0;
  rowptr[0] = 0;
  for (long e = 0; e < ctx->ncell; e++) {
    const long ix = e % nx, iy = (e / nx) % ny, iz = e / (nx * ny);
    const long cand[7] = {d == 3 && iz > 0 ? e - nx * ny : -1, iy > 0 ? e - nx : -1,
                          ix > 0 ? e - 1 : -1, e, ix + 1 < nx ? e + 1 : -1,
                          iy + 1 < ny ? e + nx : -1, d == 3 && iz + 1 < nz ? e + nx * ny : -1};
    for (int q = 0; q < 7; q++)
      if (cand[q] >= 0) {
        if (colind) colind[k] = cand[q];
        k++;
      }
    rowptr[e + 1] = k;
  }
  return PDG_OK;
}

int assemble_jacobian(pdg_context *ctx) {
  const long n = ctx->ndof;
  const int nb = ctx->nb, ns = 2 * ctx->dim + 1;
  const size_t bytes = sizeof(double) * (size_t)ctx->ncell * ns * nb * nb;
  if (!ctx->A64) PDG_CUDA_TRY(cudaMalloc(&ctx->A64, bytes));
  PDG_CUDA_TRY(cudaMemsetAsync(ctx->A64, 0, bytes, ctx->stream));
  double *x = ctx->w64[0], *y = ctx->w64[1];
  const Grid3 g = grid_of(ctx);
  int ncol = 1;
  for (int j = 0; j < ctx->dim; j++) ncol *= 3;
  const int use = ctx->use_matrix;
  ctx->use_matrix = 0;
  for (int c = 0; c < ncol; c++)
    for (int j = 0; j < nb; j++) {
      k_probe_fill<<<grid_for(n), 256, 0, ctx->stream>>>(g, ctx->ncell, nb, c, j, x);
      ApplyArgs<double> a{x, y, nullptr, 1.0, 0, 0, 0, nullptr};
      const int st = launch_apply<double>(ctx, a, ctx->K64, ctx->c64, ctx->tab64);
      if (st != PDG_OK) {
        ctx->use_matrix = use;
        return st;
      }
      k_probe_scatter<<<grid_for(n), 256, 0, ctx->stream>>>(g, ctx->ncell, nb, c, j, y, ctx->A64);
    }
  ctx->use_matrix = use;
  PDG_CUDA_TRY(cudaGetLastError());
  ctx->A_valid = 1;
  return PDG_OK;
}

int matrix_apply(pdg_context *ctx, const double *x, double *y, const double *add, double alpha,
                 int accumulate, int transpose, const int *skip) {
  if (!ctx->A_valid) return set_error(PDG_EINVAL, "the Jacobian has not been assembled");
  const Grid3 g = grid_of(ctx);
  k_bcrs_apply<<<grid_for(ctx->ndof), 256, 0, ctx->stream>>>(
      g, ctx->ncell, ctx->nb, ctx->A64, x, y, add, alpha, accumulate, transpose, skip);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

int matrix_export(pdg_context *ctx, const long *rowptr_dev, double *values_dev) {
  if (!ctx->A_valid) return set_error(PDG_EINVAL, "the Jacobian has not been assembled");
  const Grid3 g = grid_of(ctx);
  const long total = ctx->ncell * (long)ctx->nb * ctx->nb;
  k_bcrs_export<<<grid_for(total), 256, 0, ctx->stream>>>(g, ctx->ncell, ctx->nb, ctx->A64,
                                                           rowptr_dev, values_dev);
  PDG_CUDA_TRY(cudaGetLastError());
  return PDG_OK;
}

}  // namespace pdg
