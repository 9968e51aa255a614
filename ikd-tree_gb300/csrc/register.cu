// Point-to-plane scan-to-map residuals and their adjoint.
//
// The reference stops at Nearest_Search; its main consumer (FAST-LIO2) fits a
// plane through the k neighbours of every transformed scan point and
// minimises the point-to-plane residuals.  This file provides that step on
// the GPU, next to the kNN it builds on:
//
//   w_i = R(omega) p_i + t                      (scan point to map frame)
//   plane through the k neighbours of w_i:      min |A x + 1|^2,  A = [m_j^T]
//     (solved by an orthogonal factorisation, as FAST-LIO2's QR solve: the
//     normal equations square the condition number of A, which is large for
//     planes far from the origin or nearly through it)
//   n_i = x / |x|,  d_i = 1 / |x|               (plane n . q + d = 0)
//   valid_i  if every |n_i . m_j + d_i| <= plane_thresh
//   r_i = n_i . w_i + d_i,   L = 1/2 sum_valid r_i^2
// Each plane is stored as {n, d} and a point c on it (the neighbours' centroid
// projected onto the plane); residuals are evaluated as n . (w - c) in double
// from the double pose, which avoids cancelling two ~|w|-sized terms.
//
// With the neighbour sets held fixed, the planes do not depend on the pose, so
// the adjoint is closed form:
//   g_i = dL * r_i * n_i;   dL/dt = sum g_i;   dL/dp_i = R^T g_i;
//   dL/domega = J_r(omega)^T sum_i p_i x (R^T g_i)
// (J_r: right Jacobian of the SO(3) exponential).
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace ikdg {
namespace {

constexpr int RG_THREADS = 256;

__device__ __forceinline__ void transform_d(const double* Rt, double x, double y, double z, double w[3]) {
    for (int r = 0; r < 3; ++r) w[r] = Rt[3 * r] * x + Rt[3 * r + 1] * y + Rt[3 * r + 2] * z + Rt[9 + r];
}

__global__ void transform_kernel(const float* __restrict__ p, long long n, const double* __restrict__ Rt,
                                 float* __restrict__ w) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double wd[3];
    transform_d(Rt, p[3 * i], p[3 * i + 1], p[3 * i + 2], wd);
    for (int r = 0; r < 3; ++r) w[3 * i + r] = (float)wd[r];
}

// Least squares min |A x - b| for the k rows of A (k x 3) and b by a QR
// factorisation built one row at a time with Givens rotations (R upper
// triangular 3 x 3, z = Q^T b), then back substitution.  Returns false when R
// is singular.
__device__ __forceinline__ bool lsq3_givens(const float* __restrict__ rows, int k, double b_all, double x[3]) {
    double R[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double z[3] = {0, 0, 0};
    for (int j = 0; j < k; ++j) {
        double r[3] = {rows[3 * j], rows[3 * j + 1], rows[3 * j + 2]};
        double b = b_all;
        for (int c = 0; c < 3; ++c) {
            if (r[c] == 0.0) continue;
            const double h = hypot(R[c][c], r[c]);
            const double cs = R[c][c] / h, sn = r[c] / h;
            for (int m = c; m < 3; ++m) {
                const double t = cs * R[c][m] + sn * r[m];
                r[m] = -sn * R[c][m] + cs * r[m];
                R[c][m] = t;
            }
            const double t = cs * z[c] + sn * b;
            b = -sn * z[c] + cs * b;
            z[c] = t;
        }
    }
    const double scale = fmax(fabs(R[0][0]), fmax(fabs(R[1][1]), fabs(R[2][2])));
    for (int c = 0; c < 3; ++c)
        if (!(fabs(R[c][c]) > 1e-12 * scale)) return false;
    x[2] = z[2] / R[2][2];
    x[1] = (z[1] - R[1][2] * x[2]) / R[1][1];
    x[0] = (z[0] - R[0][1] * x[1] - R[0][2] * x[2]) / R[0][0];
    return true;
}

// Plane fit (least squares by Givens QR) and residual.
__global__ void plane_residual_kernel(const float* __restrict__ p, const double* __restrict__ Rt, long long n, int k,
                                      const float* __restrict__ nb, const int* __restrict__ cnt, float thresh,
                                      float4* __restrict__ planes, float* __restrict__ res, int* __restrict__ valid) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 pl = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 pc = make_float4(0.f, 0.f, 0.f, 0.f);
    int ok = 0;
    float r = 0.f;
    double xs[3];
    if (cnt[i] >= k && k >= 3 && lsq3_givens(nb + i * k * 3, k, -1.0, xs)) {
        {
            const double x0 = xs[0], x1 = xs[1], x2 = xs[2];
            const double nrm = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
            if (nrm > 0) {
                const double nx = x0 / nrm, ny = x1 / nrm, nz = x2 / nrm, dd = 1.0 / nrm;
                double cx = 0, cy = 0, cz = 0;
                ok = 1;
                for (int j = 0; j < k; ++j) {
                    const float* m = nb + (i * k + j) * 3;
                    const double e = nx * m[0] + ny * m[1] + nz * m[2] + dd;
                    if (fabs(e) > thresh) ok = 0;
                    cx += m[0];
                    cy += m[1];
                    cz += m[2];
                }
                cx /= k;
                cy /= k;
                cz /= k;
                const double off = nx * cx + ny * cy + nz * cz + dd;  // centroid -> plane
                cx -= off * nx;
                cy -= off * ny;
                cz -= off * nz;
                pl = make_float4((float)nx, (float)ny, (float)nz, (float)dd);
                pc = make_float4((float)cx, (float)cy, (float)cz, 0.f);
                if (ok) {
                    double wd[3];
                    transform_d(Rt, p[3 * i], p[3 * i + 1], p[3 * i + 2], wd);
                    r = (float)((double)pl.x * (wd[0] - (double)pc.x) + (double)pl.y * (wd[1] - (double)pc.y) +
                                (double)pl.z * (wd[2] - (double)pc.z));
                }
            }
        }
    }
    planes[2 * i] = pl;
    planes[2 * i + 1] = pc;
    res[i] = r;
    valid[i] = ok;
}

// Per block: partial sums of 1/2 r^2 (loss) over valid points.
__global__ void loss_partial_kernel(const float* __restrict__ res, const int* __restrict__ valid, long long n,
                                    double* __restrict__ partial) {
    __shared__ double sh[RG_THREADS];
    double acc = 0;
    for (long long i = (long long)blockIdx.x * RG_THREADS + threadIdx.x; i < n; i += (long long)gridDim.x * RG_THREADS)
        if (valid[i]) acc += 0.5 * (double)res[i] * (double)res[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RG_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// Adjoint: per point dL/dp_i; per block partial sums of g (for t) and
// p x (R^T g) (for omega, before J_r^T).
__global__ void adjoint_kernel(const float* __restrict__ p, long long n, const double* __restrict__ Rt,
                               const float4* __restrict__ planes, const float* __restrict__ res,
                               const int* __restrict__ valid, float dl, float* __restrict__ grad_p,
                               double* __restrict__ partial) {
    __shared__ double sh[6][RG_THREADS];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * RG_THREADS + threadIdx.x; i < n;
         i += (long long)gridDim.x * RG_THREADS) {
        double gx = 0, gy = 0, gz = 0;
        if (valid[i]) {
            const double s = (double)dl * (double)res[i];
            const float4 pl = planes[2 * i];
            gx = s * pl.x;
            gy = s * pl.y;
            gz = s * pl.z;
        }
        // v = R^T g  (Rt holds R row-major)
        const double vx = Rt[0] * gx + Rt[3] * gy + Rt[6] * gz;
        const double vy = Rt[1] * gx + Rt[4] * gy + Rt[7] * gz;
        const double vz = Rt[2] * gx + Rt[5] * gy + Rt[8] * gz;
        if (grad_p != nullptr) {
            grad_p[3 * i] = (float)vx;
            grad_p[3 * i + 1] = (float)vy;
            grad_p[3 * i + 2] = (float)vz;
        }
        const double px = p[3 * i], py = p[3 * i + 1], pz = p[3 * i + 2];
        acc[0] += gx;
        acc[1] += gy;
        acc[2] += gz;
        acc[3] += py * vz - pz * vy;
        acc[4] += pz * vx - px * vz;
        acc[5] += px * vy - py * vx;
    }
    for (int c = 0; c < 6; ++c) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int s = RG_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int c = 0; c < 6; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 6; ++c) partial[blockIdx.x * 6 + c] = sh[c][0];
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int reg_blocks(long long n) {
    long long b = (n + RG_THREADS - 1) / RG_THREADS;
    return (int)(b < 1024 ? (b > 0 ? b : 1) : 1024);
}

void launch_transform(const float* p, long long n, const double* Rt_dev, float* w, cudaStream_t s) {
    if (n <= 0) return;
    transform_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, n, Rt_dev, w);
}

void launch_plane_residual(const float* p, const double* Rt_dev, long long n, int k, const float* nb, const int* cnt,
                           float thresh, float4* planes, float* res, int* valid, double* partial, cudaStream_t s) {
    if (n <= 0) return;
    plane_residual_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, Rt_dev, n, k, nb, cnt, thresh, planes, res, valid);
    loss_partial_kernel<<<reg_blocks(n), RG_THREADS, 0, s>>>(res, valid, n, partial);
}

void launch_adjoint(const float* p, long long n, const double* Rt_dev, const float4* planes, const float* res,
                    const int* valid, float dl, float* grad_p, double* partial, cudaStream_t s) {
    if (n <= 0) return;
    adjoint_kernel<<<reg_blocks(n), RG_THREADS, 0, s>>>(p, n, Rt_dev, planes, res, valid, dl, grad_p, partial);
}

}  // namespace ikdg
