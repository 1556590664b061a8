// FP64 step kernels and FP64 read-out helpers.
//
// Compiled with --fmad=false: the FP64 step then performs exactly the
// reference's operations in the reference's order, so an FP64 parity run
// reproduces the reference's distributions bit for bit.
#include "step_kernels.cuh"

namespace lbm {

cudaError_t launch_step_f64(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t st) {
    return launch_typed<double>(Q, mode, kind, variant, p, st);
}

cudaError_t launch_multi_f64(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                              unsigned* bar, cudaStream_t st) {
    return launch_multi_typed<double>(Q, mode, even, odd, nsteps, bar, st);
}

cudaError_t init_state_f64(int Q, int what, void* f, int64_t stride, const double* fa, int64_t nact,
                           cudaStream_t st) {
    return init_typed<double>(Q, what, f, stride, fa, nact, st);
}

cudaError_t init_state(int precision, int Q, int what, void* f, int64_t stride, const double* fa, int64_t nact,
                       cudaStream_t st) {
    if (precision == P_F64) return init_state_f64(Q, what, f, stride, fa, nact, st);
    return init_state_fast(precision, Q, what, f, stride, fa, nact, st);
}

namespace {

// One block, fixed summation order: thread t adds blocks t, t+256, ... then
// a fixed shared-memory tree.  Deterministic for a given launch shape.
__global__ void k_reduce_partials(const double* __restrict__ part, int64_t nblocks, double* __restrict__ out) {
    __shared__ double red[256][kPartialStride];
    double acc[kPartialStride];
#pragma unroll
    for (int k = 0; k < kPartialStride; ++k) acc[k] = 0.0;
    for (int64_t b = threadIdx.x; b < nblocks; b += 256)
#pragma unroll
        for (int k = 0; k < kPartialStride; ++k) acc[k] += part[b * kPartialStride + k];
#pragma unroll
    for (int k = 0; k < kPartialStride; ++k) red[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int k = 0; k < kPartialStride; ++k) red[threadIdx.x][k] += red[threadIdx.x + w][k];
        __syncthreads();
    }
    if (threadIdx.x < kPartialStride) out[threadIdx.x] = red[0][threadIdx.x];
}

// f = f_eq(rho, u) + f_neq, f_neq_i = -3 tau w_i rho sum_ab (c_ia c_ib - d_ab/3) S_ab,
// S = (grad u + grad u^T)/2 from central differences (one-sided next to solid).
template <int Q>
__global__ void k_warm(const float* __restrict__ rho, const float* __restrict__ u, const int32_t* __restrict__ act_idx,
                       const int64_t* __restrict__ act_pt, int64_t nact, int nx, int ny, int nz, double tau,
                       int regularized, double* __restrict__ fa) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nact) return;
    const double r = rho[a];
    const double ux = u[3 * a], uy = u[3 * a + 1], uz = u[3 * a + 2];
    double e[Q];
    feq_all<Q, double, false>(e, r, ux, uy, uz);
    if (regularized) {
        const int64_t n = act_pt[a];
        const int idx[3] = {(int)(n % nx), (int)((n / nx) % ny), (int)(n / ((int64_t)nx * ny))};
        const int dim[3] = {nx, ny, nz};
        const int64_t step[3] = {1, nx, (int64_t)nx * ny};
        double G[3][3];  // G[b][c] = d u_c / d x_b
        for (int b = 0; b < 3; ++b) {
            int32_t ap = -1, am = -1;
            if (idx[b] + 1 < dim[b]) ap = act_idx[n + step[b]];
            if (idx[b] - 1 >= 0) am = act_idx[n - step[b]];
            for (int c = 0; c < 3; ++c) {
                const double uc = u[3 * a + c];
                double d = 0.0;
                if (ap >= 0 && am >= 0) d = 0.5 * ((double)u[3 * ap + c] - (double)u[3 * am + c]);
                else if (ap >= 0) d = (double)u[3 * ap + c] - uc;
                else if (am >= 0) d = uc - (double)u[3 * am + c];
                G[b][c] = d;
            }
        }
        for (int q = 0; q < Q; ++q) {
            const double c[3] = {(double)Lat<Q>::cx(q), (double)Lat<Q>::cy(q), (double)Lat<Q>::cz(q)};
            double s = 0.0;
            for (int b = 0; b < 3; ++b)
                for (int d = 0; d < 3; ++d) {
                    const double S = 0.5 * (G[b][d] + G[d][b]);
                    s += (c[b] * c[d] - (b == d ? 1.0 / 3.0 : 0.0)) * S;
                }
            e[q] += -3.0 * tau * Lat<Q>::w(q) * r * s;
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) fa[a * Q + q] = e[q];
}

}  // namespace

cudaError_t reduce_partials(const double* partials, int64_t nblocks, double* out, cudaStream_t st) {
    k_reduce_partials<<<1, 256, 0, st>>>(partials, nblocks, out);
    return cudaGetLastError();
}

// Next-to-wall outputs from the accumulators (w = |tau| of the last step,
// a = accumulated traction [3][n], am = accumulated |tau|): out holds
// wss[n], normal[n][3], acc[n][3], acc_mag[n], osi[n], tawss[n]
// (ComputeOSIAndTAWSS, Simulation.cpp:899-905, with pow(x, 2) as x * x).
__global__ void k_wss_out(const double* __restrict__ w, const double* __restrict__ a,
                          const double* __restrict__ am, const double* __restrict__ nrm, int64_t n, double tawss_div,
                          double* __restrict__ out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double a0 = a[p], a1 = a[n + p], a2 = a[2 * n + p], m = am[p];
    out[p] = w[p];
    double* nr = out + n;
    nr[3 * p] = nrm[p]; nr[3 * p + 1] = nrm[n + p]; nr[3 * p + 2] = nrm[2 * n + p];
    double* ac = out + 4 * n;
    ac[3 * p] = a0; ac[3 * p + 1] = a1; ac[3 * p + 2] = a2;
    out[7 * n + p] = m;
    const double norm = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
    out[8 * n + p] = 0.5 * (1.0 - (norm / m));
    out[9 * n + p] = m / tawss_div;
}

cudaError_t wss_outputs(const double* w, const double* a, const double* am, const double* nrm, int64_t n,
                        double tawss_div, double* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_wss_out<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(w, a, am, nrm, n, tawss_div, out);
    return cudaGetLastError();
}

cudaError_t warm_start_f(int Q, const float* rho, const float* u, const int32_t* act_idx, const int64_t* act_pt,
                         int64_t nact, int nx, int ny, int nz, double tau, int regularized, double* fa,
                         cudaStream_t st) {
    if (nact <= 0) return cudaSuccess;
    const unsigned g = (unsigned)ceil_div(nact, 256);
    if (Q == 19) k_warm<19><<<g, 256, 0, st>>>(rho, u, act_idx, act_pt, nact, nx, ny, nz, tau, regularized, fa);
    else k_warm<27><<<g, 256, 0, st>>>(rho, u, act_idx, act_pt, nact, nx, ny, nz, tau, regularized, fa);
    return cudaGetLastError();
}

}  // namespace lbm
