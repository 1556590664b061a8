// +z ray-parity voxelizer -- bit-identical to the reference's labelPoints.
//
// Restates, per lattice point, the reference's FP64 arithmetic in its exact
// operation order (this translation unit is compiled with --fmad=false, so
// no multiply-add is contracted, matching the reference built with
// -ffp-contract=off):
//   ray construction       ComplexGeometry.cpp:987-1035 (case 0, +z)
//   ray adjustment         ComplexGeometry.cpp:853-884
//   ray/plane test         ComplexGeometry.cpp:803-848 (uses the STL's facet normal)
//   point-in-triangle      ComplexGeometry.cpp:620-674 (recomputed normal, +z projection)
//   parity -> Fluid        ComplexGeometry.cpp:1041-1048
//
// GB300 design: the reference tests every point against every triangle
// (O(N*T)).  Here each lattice column gets a candidate list of the triangles
// whose xy extent, widened by a per-triangle margin, contains the column's
// ray; a triangle outside that widened extent provably fails the
// point-in-triangle test for every point of the column (the margin is ~1e8
// times the worst-case rounding of that test), so dropping it changes no
// count.  Triangles that can never pass (zero area, or a computed normal
// with |n_z| < 1e-16, which the reference rejects outright) are dropped;
// ill-conditioned ones go to a global list tested by every point.
// Threads run (column, k) with k fastest, so the 32 lanes of a warp walk the
// same candidate list in lock step and its triangles are broadcast loads.
#include <vector>
#include <cmath>
#include <algorithm>

#include "lbm_internal.cuh"

namespace lbm {
namespace {

struct Ray {
    double px, py, pz, ex, ey, ez;
};

__host__ __device__ inline Ray point_ray(const double* bb, const double* org, double s, int i, int j, int k) {
    double x = org[0] + i * s;
    double y = org[1] + j * s;
    double z = org[2] + k * s;
    const double rayOffset = 0.02;
    double rayLength = bb[5] - bb[4];
    Ray r;
    r.px = x; r.py = y; r.pz = z + s / 2;
    r.ex = x; r.ey = y; r.ez = z + rayLength + 0.1;
    if (r.px == bb[0]) { r.px += rayOffset; r.ex += rayOffset; }
    if (r.px == bb[1]) { r.px -= rayOffset; r.ex -= rayOffset; }
    if (r.py == bb[2]) { r.py += rayOffset; r.ey += rayOffset; }
    if (r.py == bb[3]) { r.py -= rayOffset; r.ey -= rayOffset; }
    if (r.pz == bb[4]) { r.pz += rayOffset; }
    if (r.ez == bb[5]) { r.ez -= rayOffset; }
    return r;
}

__device__ __forceinline__ bool inside_tri(double x, double y, double z, const double* __restrict__ T) {
    double x1 = T[0], y1 = T[1], z1 = T[2];
    double x2 = T[3], y2 = T[4], z2 = T[5];
    double x3 = T[6], y3 = T[7], z3 = T[8];
    double dirX = 0.0, dirY = 0.0, dirZ = 1.0;
    double uX = x2 - x1, uY = y2 - y1, uZ = z2 - z1;
    double vX = x3 - x1, vY = y3 - y1, vZ = z3 - z1;
    double nX = uY * vZ - uZ * vY;
    double nY = uZ * vX - uX * vZ;
    double nZ = uX * vY - uY * vX;
    double nLengthSq = nX * nX + nY * nY + nZ * nZ;
    const double tol = 1e-16;
    if (nLengthSq < tol * tol) return false;
    double w0X = x - x1, w0Y = y - y1, w0Z = z - z1;
    double a = -(nX * w0X + nY * w0Y + nZ * w0Z);
    double b = nX * dirX + nY * dirY + nZ * dirZ;
    if (fabs(b) < tol) return false;
    double pos = a / b;
    double ix = x + pos * dirX;
    double iy = y + pos * dirY;
    double iz = z + pos * dirZ;
    double uu = uX * uX + uY * uY + uZ * uZ;
    double uv = uX * vX + uY * vY + uZ * vZ;
    double vv = vX * vX + vY * vY + vZ * vZ;
    double wX = ix - x1, wY = iy - y1, wZ = iz - z1;
    double wu = wX * uX + wY * uY + wZ * uZ;
    double wv = wX * vX + wY * vY + wZ * vZ;
    double D = uv * uv - uu * vv;
    double sb = (uv * wv - vv * wu) / D;
    if (sb < 0.0 || sb > 1.0) return false;
    double tb = (uv * wu - uu * wv) / D;
    if (tb < 0.0 || (sb + tb) > 1.0) return false;
    return true;
}

__device__ __forceinline__ int ray_hits(const Ray& r, const double* __restrict__ T) {
    const double threshold = 1e-16;
    double dx = r.ex - r.px, dy = r.ey - r.py, dz = r.ez - r.pz;
    double nx = T[9], ny = T[10], nz = T[11];
    double qx = T[0], qy = T[1], qz = T[2];
    double numerator = (qx - r.px) * nx + (qy - r.py) * ny + (qz - r.pz) * nz;
    double denominator = dx * nx + dy * ny + dz * nz;
    if (fabs(denominator) < threshold) return 0;
    double t = numerator / denominator;
    if (t >= 0.0 && t <= 1.0) {
        double ix = r.px + t * dx;
        double iy = r.py + t * dy;
        double iz = r.pz + t * dz;
        return inside_tri(ix, iy, iz, T) ? 1 : 0;
    }
    return 0;
}

// Conservative xy margin (see file comment); -1 never counts, 1e30 never cull.
__device__ double cull_margin(const double* T, double zspan) {
    double uX = T[3] - T[0], uY = T[4] - T[1], uZ = T[5] - T[2];
    double vX = T[6] - T[0], vY = T[7] - T[1], vZ = T[8] - T[2];
    double nX = uY * vZ - uZ * vY;
    double nY = uZ * vX - uX * vZ;
    double nZ = uX * vY - uY * vX;
    double nLengthSq = nX * nX + nY * nY + nZ * nZ;
    if (nLengthSq < 1e-16 * 1e-16) return -1.0;
    if (fabs(nZ) < 1e-16) return -1.0;
    double nlen = sqrt(nLengthSq);
    double wX = vX - uX, wY = vY - uY, wZ = vZ - uZ;
    double L = sqrt(fmax(fmax(uX * uX + uY * uY + uZ * uZ, vX * vX + vY * vY + vZ * vZ), wX * wX + wY * wY + wZ * wZ));
    double cabs = 0.0;
    for (int k = 0; k < 9; ++k) cabs = fmax(cabs, fabs(T[k]));
    double shape = (L * L) / nlen;
    double m = 1e-7 * (L + zspan + cabs) * shape * shape * (nlen / fabs(nZ));
    if (!(m < 1e29)) return 1e30;
    return m;
}

struct TriBox {
    double x0, x1, y0, y1;
};

__global__ void tri_prep(const double* __restrict__ tri, int64_t ntri, double zspan, TriBox* __restrict__ box,
                         uint8_t* __restrict__ status) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const double* T = tri + 12 * t;
    double m = cull_margin(T, zspan);
    TriBox b;
    b.x0 = fmin(fmin(T[0], T[3]), T[6]) - m;
    b.x1 = fmax(fmax(T[0], T[3]), T[6]) + m;
    b.y0 = fmin(fmin(T[1], T[4]), T[7]) - m;
    b.y1 = fmax(fmax(T[1], T[4]), T[7]) + m;
    box[t] = b;
    status[t] = m < 0.0 ? 0 : (m > 1e29 ? 2 : 1);
}

// pass 0: count per column; pass 1: fill lists.
template <int PASS>
__global__ void tri_bin(int64_t ntri, const TriBox* __restrict__ box, const uint8_t* __restrict__ status,
                        const double* __restrict__ colx, const double* __restrict__ coly, int nx, int ny,
                        double ox, double oy, double s, int64_t* __restrict__ count, int32_t* __restrict__ list) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri || status[t] != 1) return;
    TriBox b = box[t];
    // clamp in FP64 before converting: margins can be far outside int range
    const double fi0 = fmax(floor((b.x0 - ox) / s) - 1.0, 0.0), fi1 = fmin(ceil((b.x1 - ox) / s) + 1.0, nx - 1.0);
    const double fj0 = fmax(floor((b.y0 - oy) / s) - 1.0, 0.0), fj1 = fmin(ceil((b.y1 - oy) / s) + 1.0, ny - 1.0);
    if (!(fi0 <= fi1) || !(fj0 <= fj1)) return;
    const int i0 = (int)fi0, i1 = (int)fi1, j0 = (int)fj0, j1 = (int)fj1;
    for (int j = j0; j <= j1; ++j) {
        double yy = coly[j];
        if (yy < b.y0 || yy > b.y1) continue;
        for (int i = i0; i <= i1; ++i) {
            double xx = colx[i];
            if (xx < b.x0 || xx > b.x1) continue;
            int64_t c = (int64_t)j * nx + i;
            if (PASS == 0) {
                atomicAdd(reinterpret_cast<unsigned long long*>(count + c), 1ull);
            } else {
                unsigned long long slot = atomicAdd(reinterpret_cast<unsigned long long*>(count + c), 1ull);
                list[slot] = (int32_t)t;
            }
        }
    }
}

struct RayParams {
    double bb[6];
    double org[3];
    double s;
    int nx, ny, nz;
    int kchunks;
};

__global__ void __launch_bounds__(128) ray_count(RayParams P, const double* __restrict__ tri,
                                                 const int64_t* __restrict__ off, const int32_t* __restrict__ list,
                                                 const int32_t* __restrict__ glob, int64_t nglob,
                                                 uint8_t* __restrict__ mask, unsigned long long* __restrict__ fluid) {
    const int64_t c = blockIdx.x / P.kchunks;
    const int k = (int)(blockIdx.x % P.kchunks) * blockDim.x + threadIdx.x;
    const int i = (int)(c % P.nx), j = (int)(c / P.nx);
    int count = 0;
    const bool live = k < P.nz;
    if (live) {
        Ray r = point_ray(P.bb, P.org, P.s, i, j, k);
        const int64_t b = off[c], e = off[c + 1];
        for (int64_t q = b; q < e; ++q) count += ray_hits(r, tri + 12 * (int64_t)__ldg(list + q));
        for (int64_t q = 0; q < nglob; ++q) count += ray_hits(r, tri + 12 * (int64_t)__ldg(glob + q));
        uint8_t v = (count % 2 == 1) ? 1 : 0;
        mask[((int64_t)k * P.ny + j) * P.nx + i] = v;
        count = v;
    }
    // block total of fluid points
    unsigned v = __reduce_add_sync(0xffffffffu, (unsigned)count);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(fluid, (unsigned long long)v);
}

#define VOX_CHECK(call)                                                        \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) {                                               \
            if (err) *err = std::string(#call) + ": " + cudaGetErrorString(_e); \
            return _e;                                                         \
        }                                                                      \
    } while (0)

}  // namespace

cudaError_t voxelize_device(const double* d_tri, int64_t ntri, const double bbox[6], const double origin[3],
                            double spacing, const int dims[3], uint8_t* d_mask, VoxResult* res, cudaStream_t st,
                            std::string* err) {
    const int nx = dims[0], ny = dims[1], nz = dims[2];
    const int64_t ncol = (int64_t)nx * ny;
    // column ray coordinates, exactly as point_ray computes them
    std::vector<double> colx(nx), coly(ny);
    for (int i = 0; i < nx; ++i) colx[i] = point_ray(bbox, origin, spacing, i, 0, 0).px;
    for (int j = 0; j < ny; ++j) coly[j] = point_ray(bbox, origin, spacing, 0, j, 0).py;
    const double zspan = (bbox[5] - bbox[4]) + 1.0 + spacing;

    TriBox* d_box = nullptr;
    uint8_t* d_status = nullptr;
    double *d_colx = nullptr, *d_coly = nullptr;
    int64_t *d_cnt = nullptr, *d_off = nullptr;
    int32_t *d_list = nullptr, *d_glob = nullptr;
    unsigned long long* d_fluid = nullptr;
    const int64_t tri_alloc = ntri > 0 ? ntri : 1;
    VOX_CHECK(cudaMallocAsync(&d_box, sizeof(TriBox) * tri_alloc, st));
    VOX_CHECK(cudaMallocAsync(&d_status, tri_alloc, st));
    VOX_CHECK(cudaMallocAsync(&d_colx, sizeof(double) * nx, st));
    VOX_CHECK(cudaMallocAsync(&d_coly, sizeof(double) * ny, st));
    VOX_CHECK(cudaMallocAsync(&d_cnt, sizeof(int64_t) * (ncol + 1), st));
    VOX_CHECK(cudaMallocAsync(&d_off, sizeof(int64_t) * (ncol + 1), st));
    VOX_CHECK(cudaMallocAsync(&d_fluid, sizeof(unsigned long long), st));
    VOX_CHECK(cudaMemcpyAsync(d_colx, colx.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, st));
    VOX_CHECK(cudaMemcpyAsync(d_coly, coly.data(), sizeof(double) * ny, cudaMemcpyHostToDevice, st));
    VOX_CHECK(cudaMemsetAsync(d_cnt, 0, sizeof(int64_t) * (ncol + 1), st));
    VOX_CHECK(cudaMemsetAsync(d_fluid, 0, sizeof(unsigned long long), st));

    const unsigned tb = 256, tg = (unsigned)ceil_div(tri_alloc, tb);
    if (ntri > 0) tri_prep<<<tg, tb, 0, st>>>(d_tri, ntri, zspan, d_box, d_status);
    VOX_CHECK(cudaGetLastError());

    // global list (ill-conditioned triangles) assembled on the host
    std::vector<uint8_t> status(ntri);
    if (ntri > 0) VOX_CHECK(cudaMemcpyAsync(status.data(), d_status, ntri, cudaMemcpyDeviceToHost, st));
    VOX_CHECK(cudaStreamSynchronize(st));
    std::vector<int32_t> glob;
    for (int64_t t = 0; t < ntri; ++t)
        if (status[t] == 2) glob.push_back((int32_t)t);
    VOX_CHECK(cudaMallocAsync(&d_glob, sizeof(int32_t) * (glob.size() + 1), st));
    if (!glob.empty())
        VOX_CHECK(cudaMemcpyAsync(d_glob, glob.data(), sizeof(int32_t) * glob.size(), cudaMemcpyHostToDevice, st));

    if (ntri > 0)
        tri_bin<0><<<tg, tb, 0, st>>>(ntri, d_box, d_status, d_colx, d_coly, nx, ny, origin[0], origin[1], spacing,
                                      d_cnt, nullptr);
    VOX_CHECK(cudaGetLastError());
    int64_t total = 0;
    VOX_CHECK(exclusive_scan_i64(d_cnt, d_off, ncol + 1, &total, st));
    VOX_CHECK(cudaMallocAsync(&d_list, sizeof(int32_t) * (total + 1), st));
    VOX_CHECK(cudaMemcpyAsync(d_cnt, d_off, sizeof(int64_t) * (ncol + 1), cudaMemcpyDeviceToDevice, st));
    if (ntri > 0)
        tri_bin<1><<<tg, tb, 0, st>>>(ntri, d_box, d_status, d_colx, d_coly, nx, ny, origin[0], origin[1], spacing,
                                      d_cnt, d_list);
    VOX_CHECK(cudaGetLastError());

    RayParams P;
    for (int q = 0; q < 6; ++q) P.bb[q] = bbox[q];
    for (int q = 0; q < 3; ++q) P.org[q] = origin[q];
    P.s = spacing;
    P.nx = nx; P.ny = ny; P.nz = nz;
    P.kchunks = (int)ceil_div(nz, 128);
    const int64_t nblocks = ncol * P.kchunks;
    if (nblocks > 0x7fffffffLL) {
        if (err) *err = "lattice too large for the voxelizer grid";
        return cudaErrorInvalidValue;
    }
    if (nblocks > 0)
        ray_count<<<(unsigned)nblocks, 128, 0, st>>>(P, d_tri, d_off, d_list, d_glob, (int64_t)glob.size(), d_mask,
                                                     d_fluid);
    VOX_CHECK(cudaGetLastError());
    unsigned long long fluid = 0;
    VOX_CHECK(cudaMemcpyAsync(&fluid, d_fluid, sizeof(fluid), cudaMemcpyDeviceToHost, st));
    VOX_CHECK(cudaStreamSynchronize(st));
    res->fluid = (int64_t)fluid;
    res->tests = (total + (int64_t)glob.size() * ncol) * nz;
    cudaFreeAsync(d_box, st);
    cudaFreeAsync(d_status, st);
    cudaFreeAsync(d_colx, st);
    cudaFreeAsync(d_coly, st);
    cudaFreeAsync(d_cnt, st);
    cudaFreeAsync(d_off, st);
    cudaFreeAsync(d_list, st);
    cudaFreeAsync(d_glob, st);
    cudaFreeAsync(d_fluid, st);
    return cudaStreamSynchronize(st);
}

}  // namespace lbm
