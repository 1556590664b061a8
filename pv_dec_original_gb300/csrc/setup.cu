// Geometry set-up on the device: node classes, boundary-node list,
// next-to-wall nodes, bulk segments and wall normals.
//
// Replaces the reference's pointer-graph construction:
//   findBoundaryPoints          ComplexGeometry.cpp:1259-1300
//   classifyBoundaryPoints      ComplexGeometry.cpp:1369-1429 (plane rules instead of PV coordinates)
//   SubDomain::CreateNodes      Subdomain.cpp:91-169 (Boundary vs Node by list membership)
//   Connectivity                Subdomain.cpp:173-197 (-> per-link "missing" bit masks)
//   IdentifyNextToWallLattices  Subdomain.cpp:201-218
//   calculateBoundaryNormals    Subdomain.cpp:224-370
// The reference links one heap object per node with shared_ptr neighbours
// and finds list membership by linear search (Utility.cpp:18-33, O(A*B));
// here a node is one class byte in a dense box and the boundary/next-to-wall
// nodes form one compact, index-sorted list built by a scan.
//
// Compiled with --fmad=false: the normals keep the reference's rounding
// (pow(d, 2) is evaluated as d*d).
#include "lbm_internal.cuh"
#include "setup.cuh"

namespace lbm {
namespace {

template <int Q>
__global__ void k_boundary(const uint8_t* __restrict__ mask, int nx, int ny, int nz, uint8_t* __restrict__ cls) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t npts = (int64_t)nx * ny * nz;
    if (n >= npts) return;
    if (!mask[n]) { cls[n] = CLS_SOLID; return; }
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    bool b = false;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int a = i + Lat<Q>::cx(q), bb = j + Lat<Q>::cy(q), c = k + Lat<Q>::cz(q);
        if (a < 0 || a >= nx || bb < 0 || bb >= ny || c < 0 || c >= nz) { b = true; break; }
        if (!mask[((int64_t)c * ny + bb) * nx + a]) { b = true; break; }
    }
    cls[n] = b ? CLS_WALL : CLS_FLUID;
}

// Extreme fluid layer per axis: ext[0..2] = min index, ext[3..5] = max index.
__global__ void k_extent(const uint8_t* __restrict__ mask, int nx, int ny, int nz, int* __restrict__ ext) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t npts = (int64_t)nx * ny * nz;
    if (n >= npts || !mask[n]) return;
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    atomicMin(ext + 0, i); atomicMin(ext + 1, j); atomicMin(ext + 2, k);
    atomicMax(ext + 3, i); atomicMax(ext + 4, j); atomicMax(ext + 5, k);
}

struct Rules {
    int n;
    int axis[LBM_MAX_BC];
    int plane[LBM_MAX_BC];
    int region[LBM_MAX_BC];
    double coord[LBM_MAX_BC], tol[LBM_MAX_BC], lo[LBM_MAX_BC][2], hi[LBM_MAX_BC][2];
    double org[3];
    double s;
};

// Plane rules match a lattice index; region rules match coordinates the way
// classifyBoundaryPoints does (ComplexGeometry.cpp:1380-1407; the reference
// compares in long double, here in FP64).  First match wins.
// The class byte records 3 + r (capped at 127 for r >= 124); bcidx holds r.
__global__ void k_classify(uint8_t* __restrict__ cls, int16_t* __restrict__ bcidx, int nx, int ny, int64_t npts,
                           Rules R) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts || cls[n] != CLS_WALL) return;
    const int idx[3] = {(int)(n % nx), (int)((n / nx) % ny), (int)(n / ((int64_t)nx * ny))};
    for (int r = 0; r < R.n; ++r) {
        const int a = R.axis[r];
        bool hit;
        if (!R.region[r]) {
            hit = idx[a] == R.plane[r];
        } else {
            const double x[3] = {R.org[0] + idx[0] * R.s, R.org[1] + idx[1] * R.s, R.org[2] + idx[2] * R.s};
            const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
            hit = fabs(x[a] - R.coord[r]) <= R.tol[r] && R.lo[r][0] < x[t1] && x[t1] < R.hi[r][0] &&
                  R.lo[r][1] < x[t2] && x[t2] < R.hi[r][1];
        }
        if (hit) {
            cls[n] = (uint8_t)(CLS_BC0 + (r < 124 ? r : 124));
            bcidx[n] = (int16_t)r;
            return;
        }
    }
}

template <int Q>
__global__ void k_next_to_wall(uint8_t* __restrict__ cls, int nx, int ny, int nz) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t npts = (int64_t)nx * ny * nz;
    if (n >= npts || cls[n] != CLS_FLUID) return;
    // an interior fluid node has all Q neighbours inside the box
    const int64_t nxy = (int64_t)nx * ny;
    bool nw = false;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int64_t m = n + Lat<Q>::cx(q) + Lat<Q>::cy(q) * (int64_t)nx + Lat<Q>::cz(q) * nxy;
        if ((cls[m] & CLS_MASK) == CLS_WALL) nw = true;
    }
    if (nw) cls[n] = CLS_FLUID | CLS_NW_BIT;
}

// Boundary-list membership, split in two: next-to-wall nodes (nwflag) and
// the other boundary-list nodes (wall and boundary-condition nodes, oflag).
__global__ void k_flag_special(const uint8_t* __restrict__ cls, int64_t npts, int64_t* __restrict__ oflag,
                               int64_t* __restrict__ nwflag) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    const uint8_t c = cls[n];
    const bool nw = (c & CLS_NW_BIT) != 0;
    oflag[n] = (!nw && (c & CLS_MASK) >= CLS_WALL) ? 1 : 0;
    nwflag[n] = nw ? 1 : 0;
}

// Boundary-list position: next-to-wall nodes first, in point order, so that
// a next-to-wall node's list entry s is also its wall-shear-stress index;
// then the other boundary-list nodes in point order.
__global__ void k_special_pos(int64_t* __restrict__ flag, int64_t* __restrict__ pos,
                              const int64_t* __restrict__ nwflag, const int64_t* __restrict__ nwpos, int64_t nnw,
                              int64_t npts) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    if (nwflag[n]) {
        flag[n] = 1;
        pos[n] = nwpos[n];
    } else if (flag[n]) {
        pos[n] = nnw + pos[n];
    }
}

__global__ void k_scatter(const int64_t* __restrict__ flag, const int64_t* __restrict__ pos, int64_t npts,
                          int64_t* __restrict__ out) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts || !flag[n]) return;
    out[pos[n]] = n;
}

template <int Q>
__global__ void k_special_info(const int64_t* __restrict__ sp_pt, int64_t nsp, const uint8_t* __restrict__ cls,
                               const int64_t* __restrict__ nwpos, int nx, int ny, int nz,
                               const int16_t* __restrict__ bcidx, uint32_t* __restrict__ miss,
                               uint8_t* __restrict__ spc, int32_t* __restrict__ spnw, int32_t* __restrict__ spbc,
                               double* __restrict__ prof, ProfileSpec ps) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsp) return;
    const int64_t n = sp_pt[s];
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    uint32_t m = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int a = i + Lat<Q>::cx(q), b = j + Lat<Q>::cy(q), c = k + Lat<Q>::cz(q);
        bool missing = (a < 0 || a >= nx || b < 0 || b >= ny || c < 0 || c >= nz) ||
                       cls[((int64_t)c * ny + b) * nx + a] == CLS_SOLID;
        if (missing) m |= 1u << q;
    }
    miss[s] = m;
    const uint8_t c = cls[n];
    spc[s] = c & CLS_MASK;
    spnw[s] = (c & CLS_NW_BIT) ? (int32_t)nwpos[n] : -1;
    const bool is_bc = (c & CLS_MASK) >= CLS_BC0;
    const int b = is_bc ? (int)bcidx[n] : -1;
    spbc[s] = b;
    double p = 0.0;
    if (is_bc && b < ps.n) {
        if (ps.profile[b] == 0) {
            p = 1.0;
        } else {
            // same expression as the reference harness / oracle profile factor
            const double xyz[3] = {ps.org[0] + i * ps.s, ps.org[1] + j * ps.s, ps.org[2] + k * ps.s};
            const int a = ps.axis[b];
            const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
            double d1 = xyz[t1] - ps.c1[b], d2 = xyz[t2] - ps.c2[b];
            double v = 1.0 - (d1 * d1 + d2 * d2) / (ps.R[b] * ps.R[b]);
            p = v > 0.0 ? v : 0.0;
        }
    }
    prof[s] = p;
}

__global__ void k_active_flags(const uint8_t* __restrict__ cls, int64_t npts, int64_t* __restrict__ flag) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    flag[n] = cls[n] != CLS_SOLID ? 1 : 0;
}

// Per active node: index maps and the step kernel's packed word
// (segment | special << 31 | missing mask << 32 | class << 59 | next-to-wall << 63).
template <int Q>
__global__ void k_active_index(const int64_t* __restrict__ flag, const int64_t* __restrict__ pos,
                               const int64_t* __restrict__ spflag, const int64_t* __restrict__ sppos,
                               const uint8_t* __restrict__ cls, int nx, int ny, int nz,
                               const int32_t* __restrict__ seg_of_act, int32_t* __restrict__ act_idx,
                               int64_t* __restrict__ act_pt,
                               uint64_t* __restrict__ act_word, int32_t* __restrict__ sp_of_act) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t npts = (int64_t)nx * ny * nz;
    if (n >= npts) return;
    if (!flag[n]) {
        act_idx[n] = -1;
        return;
    }
    const int64_t a = pos[n];
    act_idx[n] = (int32_t)a;
    act_pt[a] = n;
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    uint64_t miss = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int x = i + Lat<Q>::cx(q), y = j + Lat<Q>::cy(q), z = k + Lat<Q>::cz(q);
        bool m = (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) ||
                 cls[((int64_t)z * ny + y) * nx + x] == CLS_SOLID;
        if (m) miss |= 1ull << q;
    }
    const uint8_t c = cls[n];
    const bool sp = spflag[n] != 0;
    act_word[a] = (uint64_t)(uint32_t)seg_of_act[a] | ((uint64_t)sp << 31) | (miss << 32) |
                  ((uint64_t)((c & CLS_MASK) < CLS_BC0 ? (c & CLS_MASK) : CLS_BC0) << 59) |
                  ((uint64_t)((c & CLS_NW_BIT) ? 1 : 0) << 63);
    sp_of_act[a] = sp ? (int32_t)sppos[n] : -1;
}

// Per-triangle unit normal, area and centroid (Subdomain.cpp:244-267).
__global__ void k_tri_weights(const double* __restrict__ tri, int64_t ntri, double* __restrict__ tw) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const double* T = tri + 12 * t;
    double ux = T[3] - T[0], uy = T[4] - T[1], uz = T[5] - T[2];
    double vx = T[6] - T[0], vy = T[7] - T[1], vz = T[8] - T[2];
    double nx = uy * vz - uz * vy;
    double ny = uz * vx - ux * vz;
    double nz = ux * vy - uy * vx;
    double norm = sqrt(nx * nx + ny * ny + nz * nz);
    if (norm > 0) { nx /= norm; ny /= norm; nz /= norm; }
    double area = 0.5 * norm;
    double* o = tw + 7 * t;
    o[0] = nx; o[1] = ny; o[2] = nz; o[3] = area;
    o[4] = (T[0] + T[3] + T[6]) / 3.0;
    o[5] = (T[1] + T[4] + T[7]) / 3.0;
    o[6] = (T[2] + T[5] + T[8]) / 3.0;
}

constexpr int kNormThreads = 128;
constexpr int kNormTile = 256;

__global__ void __launch_bounds__(kNormThreads) k_normals(const double* __restrict__ tw, int64_t ntri,
                                                         const int64_t* __restrict__ pts, int64_t npts, int nx,
                                                         int ny, double ox, double oy, double oz, double s,
                                                         double* __restrict__ out) {
    __shared__ double tile[kNormTile * 7];
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double x = 0, y = 0, z = 0;
    if (p < npts) {
        const int64_t n = pts[p];
        const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
        x = ox + i * s; y = oy + j * s; z = oz + k * s;
    }
    double n0 = 0.0, n1 = 0.0, n2 = 0.0;
    for (int64_t t0 = 0; t0 < ntri; t0 += kNormTile) {
        const int cnt = (int)min((int64_t)kNormTile, ntri - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt * 7; e += blockDim.x) tile[e] = tw[7 * t0 + e];
        __syncthreads();
        for (int t = 0; t < cnt; ++t) {
            const double* o = tile + 7 * t;
            double dx = x - o[4], dy = y - o[5], dz = z - o[6];
            // area / distance^2 straight from the squared distance (the
            // reference squares the square root: the two differ by an
            // ulp or so per term, far below the normals' 1e-13 checks,
            // and the FP64 square root of every pair goes)
            double w = o[3] / (dx * dx + dy * dy + dz * dz);
            n0 += o[0] * w;
            n1 += o[1] * w;
            n2 += o[2] * w;
        }
    }
    if (p < npts) {
        double norm = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
        if (norm > 0) { n0 /= norm; n1 /= norm; n2 /= norm; }
        out[p] = n0;
        out[npts + p] = n1;
        out[2 * npts + p] = n2;
    }
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)ceil_div(n > 0 ? n : 1, t); }

}  // namespace

#define SETUP_CHECK(call)                                                       \
    do {                                                                        \
        cudaError_t _e = (call);                                                \
        if (_e != cudaSuccess) {                                                \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);          \
            return _e;                                                          \
        }                                                                       \
    } while (0)

cudaError_t build_geometry(int Q, const uint8_t* d_mask, int nx, int ny, int nz, const lbm_bc_spec* bc, int nbc,
                           const double origin[3], double spacing, const int32_t* d_seg_of_act, GeometryLists& out,
                           cudaStream_t st, std::string& err) {
    const int64_t npts = (int64_t)nx * ny * nz;
    out.npts = npts;
    // padded to whole 32-point segments: the bulk kernel reads the class
    // byte of every lane of a segment
    const int64_t npad = ceil_div(npts, 32) * 32;
    SETUP_CHECK(cudaMallocAsync(&out.cls, npad, st));
    SETUP_CHECK(cudaMemsetAsync(out.cls, 0, npad, st));
    if (Q == 19) k_boundary<19><<<blocks(npts), 256, 0, st>>>(d_mask, nx, ny, nz, out.cls);
    else k_boundary<27><<<blocks(npts), 256, 0, st>>>(d_mask, nx, ny, nz, out.cls);
    SETUP_CHECK(cudaGetLastError());

    // plane rules; plane -1 = extreme fluid layer on the face
    Rules R{};
    R.n = nbc;
    bool need_ext = false;
    for (int b = 0; b < nbc; ++b) need_ext |= bc[b].plane < 0 && !bc[b].region;
    int ext[6] = {0, 0, 0, -1, -1, -1};
    if (need_ext) {
        int* d_ext = nullptr;
        int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, -1, -1, -1};
        SETUP_CHECK(cudaMallocAsync(&d_ext, sizeof(init), st));
        SETUP_CHECK(cudaMemcpyAsync(d_ext, init, sizeof(init), cudaMemcpyHostToDevice, st));
        k_extent<<<blocks(npts), 256, 0, st>>>(d_mask, nx, ny, nz, d_ext);
        SETUP_CHECK(cudaMemcpyAsync(ext, d_ext, sizeof(ext), cudaMemcpyDeviceToHost, st));
        SETUP_CHECK(cudaStreamSynchronize(st));
        cudaFreeAsync(d_ext, st);
    }
    R.org[0] = origin[0]; R.org[1] = origin[1]; R.org[2] = origin[2];
    R.s = spacing;
    for (int b = 0; b < nbc; ++b) {
        const int face = bc[b].face;
        R.axis[b] = face / 2;
        R.plane[b] = bc[b].plane >= 0 ? bc[b].plane : (face % 2 == 0 ? ext[face / 2] : ext[3 + face / 2]);
        R.region[b] = bc[b].region;
        R.coord[b] = bc[b].coord;
        R.tol[b] = bc[b].tol;
        for (int t = 0; t < 2; ++t) { R.lo[b][t] = bc[b].lo[t]; R.hi[b][t] = bc[b].hi[t]; }
        out.plane[b] = R.plane[b];
    }
    SETUP_CHECK(cudaMallocAsync(&out.bcidx, sizeof(int16_t) * npad, st));
    k_classify<<<blocks(npts), 256, 0, st>>>(out.cls, out.bcidx, nx, ny, npts, R);
    SETUP_CHECK(cudaGetLastError());
    if (Q == 19) k_next_to_wall<19><<<blocks(npts), 256, 0, st>>>(out.cls, nx, ny, nz);
    else k_next_to_wall<27><<<blocks(npts), 256, 0, st>>>(out.cls, nx, ny, nz);
    SETUP_CHECK(cudaGetLastError());

    // compact lists
    int64_t *flag = nullptr, *pos = nullptr, *nwflag = nullptr, *nwpos = nullptr;
    SETUP_CHECK(cudaMallocAsync(&flag, sizeof(int64_t) * npts, st));
    SETUP_CHECK(cudaMallocAsync(&pos, sizeof(int64_t) * npts, st));
    SETUP_CHECK(cudaMallocAsync(&nwflag, sizeof(int64_t) * npts, st));
    SETUP_CHECK(cudaMallocAsync(&nwpos, sizeof(int64_t) * npts, st));
    k_flag_special<<<blocks(npts), 256, 0, st>>>(out.cls, npts, flag, nwflag);
    int64_t nother = 0;
    SETUP_CHECK(exclusive_scan_i64(flag, pos, npts, &nother, st));
    SETUP_CHECK(exclusive_scan_i64(nwflag, nwpos, npts, &out.nnw, st));
    out.nsp = out.nnw + nother;
    k_special_pos<<<blocks(npts), 256, 0, st>>>(flag, pos, nwflag, nwpos, out.nnw, npts);
    SETUP_CHECK(cudaGetLastError());
    SETUP_CHECK(cudaMallocAsync(&out.sp_pt, sizeof(int64_t) * (out.nsp + 1), st));
    SETUP_CHECK(cudaMallocAsync(&out.nw_pt, sizeof(int64_t) * (out.nnw + 1), st));
    k_scatter<<<blocks(npts), 256, 0, st>>>(flag, pos, npts, out.sp_pt);
    k_scatter<<<blocks(npts), 256, 0, st>>>(nwflag, nwpos, npts, out.nw_pt);
    SETUP_CHECK(cudaGetLastError());
    SETUP_CHECK(cudaMallocAsync(&out.sp_miss, sizeof(uint32_t) * (out.nsp + 1), st));
    SETUP_CHECK(cudaMallocAsync(&out.sp_cls, out.nsp + 1, st));
    SETUP_CHECK(cudaMallocAsync(&out.sp_nw, sizeof(int32_t) * (out.nsp + 1), st));
    SETUP_CHECK(cudaMallocAsync(&out.sp_bc, sizeof(int32_t) * (out.nsp + 1), st));
    SETUP_CHECK(cudaMallocAsync(&out.sp_prof, sizeof(double) * (out.nsp + 1), st));
    ProfileSpec ps{};
    ps.n = nbc;
    ps.s = spacing;
    for (int d = 0; d < 3; ++d) ps.org[d] = origin[d];
    for (int b = 0; b < nbc; ++b) {
        ps.profile[b] = bc[b].profile;
        ps.axis[b] = bc[b].face / 2;
        ps.c1[b] = bc[b].c1; ps.c2[b] = bc[b].c2; ps.R[b] = bc[b].R;
    }
    if (out.nsp > 0) {
        if (Q == 19)
            k_special_info<19><<<blocks(out.nsp), 256, 0, st>>>(out.sp_pt, out.nsp, out.cls, nwpos, nx, ny, nz,
                                                               out.bcidx, out.sp_miss, out.sp_cls, out.sp_nw,
                                                               out.sp_bc, out.sp_prof, ps);
        else
            k_special_info<27><<<blocks(out.nsp), 256, 0, st>>>(out.sp_pt, out.nsp, out.cls, nwpos, nx, ny, nz,
                                                               out.bcidx, out.sp_miss, out.sp_cls, out.sp_nw,
                                                               out.sp_bc, out.sp_prof, ps);
        SETUP_CHECK(cudaGetLastError());
    }

    // active index and the packed per-node words of the step kernel
    int64_t *aflag = nullptr, *apos = nullptr;
    SETUP_CHECK(cudaMallocAsync(&aflag, sizeof(int64_t) * npts, st));
    SETUP_CHECK(cudaMallocAsync(&apos, sizeof(int64_t) * npts, st));
    k_active_flags<<<blocks(npts), 256, 0, st>>>(out.cls, npts, aflag);
    SETUP_CHECK(exclusive_scan_i64(aflag, apos, npts, &out.nact, st));
    SETUP_CHECK(cudaMallocAsync(&out.act_idx, sizeof(int32_t) * npts, st));
    SETUP_CHECK(cudaMallocAsync(&out.act_pt, sizeof(int64_t) * (out.nact + 1), st));
    SETUP_CHECK(cudaMallocAsync(&out.act_word, sizeof(uint64_t) * (out.nact + 1), st));
    // padded: the tiled step kernel copies whole 16-byte groups
    SETUP_CHECK(cudaMallocAsync(&out.sp_of_act, sizeof(int32_t) * (out.nact + 4), st));
    if (Q == 19)
        k_active_index<19><<<blocks(npts), 256, 0, st>>>(aflag, apos, flag, pos, out.cls, nx, ny, nz, d_seg_of_act,
                                                         out.act_idx, out.act_pt, out.act_word, out.sp_of_act);
    else
        k_active_index<27><<<blocks(npts), 256, 0, st>>>(aflag, apos, flag, pos, out.cls, nx, ny, nz, d_seg_of_act,
                                                         out.act_idx, out.act_pt, out.act_word, out.sp_of_act);
    SETUP_CHECK(cudaGetLastError());
    cudaFreeAsync(aflag, st);
    cudaFreeAsync(apos, st);
    cudaFreeAsync(flag, st);
    cudaFreeAsync(pos, st);
    cudaFreeAsync(nwflag, st);
    cudaFreeAsync(nwpos, st);
    SETUP_CHECK(cudaStreamSynchronize(st));
    return cudaSuccess;
}

// Nearest next-to-wall node of each query point (the lattice carries WSS,
// OSI and TAWSS on those nodes).  With g the point in lattice units and c =
// round(g), the cube of half-width R around c holds every lattice point
// closer than R + 0.5; the cube grows (R = 1, 2, 4, ...) until the best
// node found lies within that bound, so the result is the exact nearest
// (ties to the lower next-to-wall index), or -1 beyond rmax.
__global__ void k_nearest_nw(const double* __restrict__ xyz, int64_t nv, const int32_t* __restrict__ act_idx,
                             const int32_t* __restrict__ sp_of_act, int64_t nnw, int nx, int ny, int nz, double ox,
                             double oy, double oz, double sp, int rmax, int64_t* __restrict__ out_idx,
                             double* __restrict__ out_dist) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const double g[3] = {(xyz[3 * v] - ox) / sp, (xyz[3 * v + 1] - oy) / sp, (xyz[3 * v + 2] - oz) / sp};
    const int dims[3] = {nx, ny, nz};
    int c[3];
    for (int d = 0; d < 3; ++d) {
        double r = rint(g[d]);
        r = r < 0.0 ? 0.0 : (r > dims[d] - 1 ? (double)(dims[d] - 1) : r);
        c[d] = (int)r;
    }
    int64_t best = -1;
    double best_d2 = 0.0;
    for (int R = 1; R <= rmax; R *= 2) {
        const int lo[3] = {max(c[0] - R, 0), max(c[1] - R, 0), max(c[2] - R, 0)};
        const int hi[3] = {min(c[0] + R, nx - 1), min(c[1] + R, ny - 1), min(c[2] + R, nz - 1)};
        for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int i = lo[0]; i <= hi[0]; ++i) {
                    const int32_t a = act_idx[((int64_t)k * ny + j) * nx + i];
                    if (a < 0) continue;
                    const int32_t e = sp_of_act[a];
                    if (e < 0 || e >= nnw) continue;
                    const double dx = i - g[0], dy = j - g[1], dz = k - g[2];
                    const double d2 = dx * dx + dy * dy + dz * dz;
                    if (best < 0 || d2 < best_d2 || (d2 == best_d2 && e < best)) {
                        best = e;
                        best_d2 = d2;
                    }
                }
        if (best >= 0 && sqrt(best_d2) <= R + 0.5) break;
    }
    out_idx[v] = best;
    if (out_dist) out_dist[v] = best >= 0 ? sqrt(best_d2) * sp : -1.0;
}

cudaError_t nearest_next_to_wall(const double* d_xyz, int64_t nv, const GeometryLists& g, int nx, int ny, int nz,
                                 const double origin[3], double spacing, int rmax, int64_t* d_idx, double* d_dist,
                                 cudaStream_t st) {
    if (nv <= 0) return cudaSuccess;
    k_nearest_nw<<<blocks(nv, 128), 128, 0, st>>>(d_xyz, nv, g.act_idx, g.sp_of_act, g.nnw, nx, ny, nz, origin[0],
                                                 origin[1], origin[2], spacing, rmax, d_idx, d_dist);
    return cudaGetLastError();
}

// Wall distance of every missing link of the boundary list, for the
// interpolated bounce-back: for entry s and arriving population q whose
// source x - c_q (= x + c_i, i = opp q) is not active, the fraction t in
// [0, 1] along the link x -> x + c_i at which it first meets a triangle
// (segment-triangle intersection after Moller and Trumbore, 1997, in FP64),
// stored as q[qi * nsp + s]; 0.5 (half-way) where no link is missing or no
// triangle crosses it.  Triangles are tested in file order; the smallest t
// wins.  tri: ntri rows of x1 y1 z1 x2 y2 z2 x3 y3 z3 nx ny nz.
__device__ __forceinline__ bool seg_tri(const double* P0, const double* d, const double* T, double& t) {
    const double e1[3] = {T[3] - T[0], T[4] - T[1], T[5] - T[2]};
    const double e2[3] = {T[6] - T[0], T[7] - T[1], T[8] - T[2]};
    const double pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
    const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
    if (fabs(det) < 1e-300) return false;
    const double inv = 1.0 / det;
    const double tv[3] = {P0[0] - T[0], P0[1] - T[1], P0[2] - T[2]};
    const double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
    const double v = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) * inv;
    if (v < 0.0 || u + v > 1.0) return false;
    t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
    return t >= 0.0 && t <= 1.0;
}

template <int Q>
__global__ void k_wall_q(const int64_t* __restrict__ sp_pt, const uint32_t* __restrict__ sp_miss, int64_t nsp,
                         int nx, int ny, double ox, double oy, double oz, double sp, const double* __restrict__ tri,
                         int64_t ntri, float* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nsp) return;
    const int64_t n = sp_pt[e];
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    const double P0[3] = {ox + i * sp, oy + j * sp, oz + k * sp};
    const uint32_t miss = sp_miss[e];
    for (int q = 0; q < Q; ++q) {
        float qw = 0.5f;
        const int ci = Lat<Q>::opp(q);
        if ((miss >> ci) & 1u) {
            const double d[3] = {Lat<Q>::cx(ci) * sp, Lat<Q>::cy(ci) * sp, Lat<Q>::cz(ci) * sp};
            const double lo[3] = {fmin(P0[0], P0[0] + d[0]), fmin(P0[1], P0[1] + d[1]), fmin(P0[2], P0[2] + d[2])};
            const double hi[3] = {fmax(P0[0], P0[0] + d[0]), fmax(P0[1], P0[1] + d[1]), fmax(P0[2], P0[2] + d[2])};
            double best = 2.0;
            for (int64_t r = 0; r < ntri; ++r) {
                const double* T = tri + 12 * r;
                // bounding-box rejection (exact: a hit lies in both boxes)
                if (fmax(T[0], fmax(T[3], T[6])) < lo[0] || fmin(T[0], fmin(T[3], T[6])) > hi[0] ||
                    fmax(T[1], fmax(T[4], T[7])) < lo[1] || fmin(T[1], fmin(T[4], T[7])) > hi[1] ||
                    fmax(T[2], fmax(T[5], T[8])) < lo[2] || fmin(T[2], fmin(T[5], T[8])) > hi[2])
                    continue;
                double t;
                if (seg_tri(P0, d, T, t) && t < best) best = t;
            }
            if (best <= 1.0) qw = (float)best;
        }
        out[(int64_t)q * nsp + e] = qw;
    }
}

cudaError_t wall_distances(int Q, const double* d_tri, int64_t ntri, const GeometryLists& g, int nx, int ny,
                           const double origin[3], double spacing, float* d_q, cudaStream_t st) {
    if (g.nsp <= 0) return cudaSuccess;
    if (Q == 19)
        k_wall_q<19><<<blocks(g.nsp, 128), 128, 0, st>>>(g.sp_pt, g.sp_miss, g.nsp, nx, ny, origin[0], origin[1],
                                                        origin[2], spacing, d_tri, ntri, d_q);
    else
        k_wall_q<27><<<blocks(g.nsp, 128), 128, 0, st>>>(g.sp_pt, g.sp_miss, g.nsp, nx, ny, origin[0], origin[1],
                                                        origin[2], spacing, d_tri, ntri, d_q);
    return cudaGetLastError();
}

cudaError_t surface_normals(const double* d_tri, int64_t ntri, const int64_t* d_pts, int64_t npts, int nx, int ny,
                            const double origin[3], double spacing, double* d_out, cudaStream_t st) {
    if (npts <= 0) return cudaSuccess;
    double* tw = nullptr;
    cudaError_t e = cudaMallocAsync(&tw, sizeof(double) * 7 * (ntri > 0 ? ntri : 1), st);
    if (e != cudaSuccess) return e;
    if (ntri > 0) k_tri_weights<<<blocks(ntri), 256, 0, st>>>(d_tri, ntri, tw);
    k_normals<<<blocks(npts, kNormThreads), kNormThreads, 0, st>>>(tw, ntri, d_pts, npts, nx, ny, origin[0],
                                                                  origin[1], origin[2], spacing, d_out);
    e = cudaGetLastError();
    cudaFreeAsync(tw, st);
    return e;
}

}  // namespace lbm
