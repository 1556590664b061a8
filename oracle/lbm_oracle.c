/*
 * CPU restatement of the reference's hot path -- TEST INFRASTRUCTURE ONLY.
 * (Header: lbm_oracle.h.)  Compiled with -ffp-contract=off; every
 * floating-point expression keeps the reference's evaluation order so that
 * results agree bit for bit with the reference built the same way.
 *
 * Restated reference code:
 *   LatticeModel.cpp:51-151, 208-334   lattice tables
 *   ComplexGeometry.cpp:145-165        bounding box and lattice size
 *   ComplexGeometry.cpp:978-1053       labelPoints (ray construction)
 *   ComplexGeometry.cpp:853-884        adjustLineCoordinates (+z case)
 *   ComplexGeometry.cpp:803-848        countIntersectinsTriangle
 *   ComplexGeometry.cpp:620-674        isPointInsideTriangle
 *   ComplexGeometry.cpp:1259-1300      findBoundaryPoints
 *   Subdomain.cpp:173-218              Connectivity, IdentifyNextToWallLattices
 *   Subdomain.cpp:224-370              calculateBoundaryNormals
 *   Node.cpp:30-37                     Initialize (f = w, fnew = 0)
 *   Simulation.cpp:43-208              Collision
 *   Simulation.cpp:211-237             Streaming (push, zero skip)
 *   Boundary.cpp:129-157               ApplyBc (Zou-He velocity, x-min)
 *   Simulation.cpp:628-838             ApplyOutletBc (y-max, z-min)
 *   Simulation.cpp:843-863             ApplyWallBc
 *   Simulation.cpp:880-905             ComputeWallShearStress, ComputeOSIAndTAWSS
 * The physics mode (half-way bounce-back, Zou-He on any face, stress with the
 * (1 - 1/2tau) factor) has no reference counterpart; it restates the
 * library's own documented semantics.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* lattice tables */

static const int C19[19][3] = {
    {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0},
    {-1, 0, 1}, {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1}, {0, 0, 0}};
static const int OPP19[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};

static const int C27[27][3] = {
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, 0, 1}, {-1, 0, 1}, {1, 0, -1},
    {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1}, {1, 1, 1}, {-1, -1, -1},
    {1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {-1, 1, -1}, {1, -1, -1}, {-1, 1, 1}};
static const int OPP27[27] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15,
                              20, 19, 22, 21, 24, 23, 26, 25};

static double weight(int Q, int q) {
    if (Q == 19) {
        if (q < 6) return 2.0 / 36.0;
        if (q < 18) return 1.0 / 36.0;
        return 12.0 / 36.0;
    }
    if (q == 0) return 8.0 / 27.0;
    if (q < 7) return 2.0 / 27.0;
    if (q < 19) return 1.0 / 54.0;
    return 1.0 / 216.0;
}

static const int* cvec(int Q, int q) { return Q == 19 ? C19[q] : C27[q]; }
static int opp_of(int Q, int q) { return Q == 19 ? OPP19[q] : OPP27[q]; }

int oracle_lattice(int Q, int* c, double* w, int* opp) {
    if (Q != 19 && Q != 27) return -1;
    for (int q = 0; q < Q; ++q) {
        for (int d = 0; d < 3; ++d) c[3 * q + d] = cvec(Q, q)[d];
        w[q] = weight(Q, q);
        opp[q] = opp_of(Q, q);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* geometry */

static double dmin(double a, double b) { return b < a ? b : a; }
static double dmax(double a, double b) { return a < b ? b : a; }

void oracle_bbox_dims(const double* t, int64_t ntri, double spacing, double* bb, int* dims) {
    double mnx = INFINITY, mny = INFINITY, mnz = INFINITY;
    double mxx = -INFINITY, mxy = -INFINITY, mxz = -INFINITY;
    for (int64_t k = 0; k < ntri; ++k) {
        const double* r = t + 12 * k;
        /* y and z ignore the third vertex (ComplexGeometry.cpp:147-151) */
        mnx = dmin(dmin(dmin(mnx, r[0]), r[3]), r[6]);
        mny = dmin(dmin(mny, r[1]), r[4]);
        mnz = dmin(dmin(mnz, r[2]), r[5]);
        mxx = dmax(dmax(dmax(mxx, r[0]), r[3]), r[6]);
        mxy = dmax(dmax(mxy, r[1]), r[4]);
        mxz = dmax(dmax(mxz, r[2]), r[5]);
    }
    bb[0] = mnx; bb[1] = mxx; bb[2] = mny; bb[3] = mxy; bb[4] = mnz; bb[5] = mxz;
    dims[0] = (int)ceil((mxx - mnx) / spacing) + 1;
    dims[1] = (int)ceil((mxy - mny) / spacing) + 1;
    dims[2] = (int)ceil((mxz - mnz) / spacing);
}

/* isPointInsideTriangle (ComplexGeometry.cpp:620-674), +z projection. */
static int inside_tri(double x, double y, double z, const double* T) {
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
    if (nLengthSq < tol * tol) return 0;
    double w0X = x - x1, w0Y = y - y1, w0Z = z - z1;
    double a = -(nX * w0X + nY * w0Y + nZ * w0Z);
    double b = nX * dirX + nY * dirY + nZ * dirZ;
    if (fabs(b) < tol) return 0;
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
    double s = (uv * wv - vv * wu) / D;
    if (s < 0.0 || s > 1.0) return 0;
    double t = (uv * wu - uu * wv) / D;
    if (t < 0.0 || (s + t) > 1.0) return 0;
    return 1;
}

/* One triangle of countIntersectinsTriangle (ComplexGeometry.cpp:807-844). */
static int ray_hits(double px, double py, double pz, double ex, double ey, double ez, const double* T) {
    const double threshold = 1e-16;
    double dx = ex - px, dy = ey - py, dz = ez - pz;
    double nx = T[9], ny = T[10], nz = T[11];
    double qx = T[0], qy = T[1], qz = T[2];
    double numerator = (qx - px) * nx + (qy - py) * ny + (qz - pz) * nz;
    double denominator = dx * nx + dy * ny + dz * nz;
    if (fabs(denominator) < threshold) return 0;
    double t = numerator / denominator;
    if (t >= 0.0 && t <= 1.0) {
        double ix = px + t * dx;
        double iy = py + t * dy;
        double iz = pz + t * dz;
        return inside_tri(ix, iy, iz, T);
    }
    return 0;
}

/* Ray of labelPoints (+z) after adjustLineCoordinates case 0. */
static void point_ray(const double* bb, const double* org, double s, int i, int j, int k,
                      double* p, double* e) {
    double x = org[0] + i * s;
    double y = org[1] + j * s;
    double z = org[2] + k * s;
    const double rayOffset = 0.02;
    double rayLength = bb[5] - bb[4];
    p[0] = x; p[1] = y; p[2] = z + s / 2;
    e[0] = x; e[1] = y; e[2] = z + rayLength + 0.1;
    if (p[0] == bb[0]) { p[0] += rayOffset; e[0] += rayOffset; }
    if (p[0] == bb[1]) { p[0] -= rayOffset; e[0] -= rayOffset; }
    if (p[1] == bb[2]) { p[1] += rayOffset; e[1] += rayOffset; }
    if (p[1] == bb[3]) { p[1] -= rayOffset; e[1] -= rayOffset; }
    if (p[2] == bb[4]) { p[2] += rayOffset; }
    if (e[2] == bb[5]) { e[2] -= rayOffset; }
}

double oracle_cull_margin(const double* T, double zspan) {
    double uX = T[3] - T[0], uY = T[4] - T[1], uZ = T[5] - T[2];
    double vX = T[6] - T[0], vY = T[7] - T[1], vZ = T[8] - T[2];
    double nX = uY * vZ - uZ * vY;
    double nY = uZ * vX - uX * vZ;
    double nZ = uX * vY - uY * vX;
    double nLengthSq = nX * nX + nY * nY + nZ * nZ;
    if (nLengthSq < 1e-16 * 1e-16) return -1.0;  /* isPointInsideTriangle always false */
    if (fabs(nZ) < 1e-16) return -1.0;           /* b == nZ exactly: always false */
    double nlen = sqrt(nLengthSq);
    double wX = vX - uX, wY = vY - uY, wZ = vZ - uZ;
    double L = sqrt(dmax(dmax(uX * uX + uY * uY + uZ * uZ, vX * vX + vY * vY + vZ * vZ),
                         wX * wX + wY * wY + wZ * wZ));
    double cabs = 0.0;
    for (int k = 0; k < 9; ++k) cabs = dmax(cabs, fabs(T[k]));
    double shape = (L * L) / nlen;
    double m = 1e-7 * (L + zspan + cabs) * shape * shape * (nlen / fabs(nZ));
    if (!(m < 1e29)) return 1e30;
    return m;
}

int64_t oracle_voxelize(const double* tri, int64_t ntri, const double* bb, const double* org, double s,
                        const int* dims, uint8_t* mask, int culled, int nthreads) {
    const int nx = dims[0], ny = dims[1], nz = dims[2];
    const int64_t ncol = (int64_t)nx * ny;
    int64_t* off = NULL;
    int32_t* lst = NULL;
    int32_t* glob = NULL;
    int64_t nglob = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (culled) {
        /* Column candidate lists: triangle T is kept for column (i,j) when
         * the column's ray lies inside T's xy extent widened by its margin. */
        double zspan = (bb[5] - bb[4]) + 1.0 + s;
        double* marg = (double*)malloc(sizeof(double) * (size_t)(ntri > 0 ? ntri : 1));
        double* colx = (double*)malloc(sizeof(double) * (size_t)nx);
        double* coly = (double*)malloc(sizeof(double) * (size_t)ny);
        for (int i = 0; i < nx; ++i) {
            double p[3], e[3];
            point_ray(bb, org, s, i, 0, 0, p, e);
            colx[i] = p[0];
        }
        for (int j = 0; j < ny; ++j) {
            double p[3], e[3];
            point_ray(bb, org, s, 0, j, 0, p, e);
            coly[j] = p[1];
        }
        glob = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntri > 0 ? ntri : 1));
        off = (int64_t*)calloc((size_t)ncol + 1, sizeof(int64_t));
        for (int64_t t = 0; t < ntri; ++t) {
            marg[t] = oracle_cull_margin(tri + 12 * t, zspan);
            if (marg[t] > 1e29) glob[nglob++] = (int32_t)t;
        }
        for (int pass = 0; pass < 2; ++pass) {
            int64_t* cur = NULL;
            if (pass == 1) {
                for (int64_t c = 0; c < ncol; ++c) off[c + 1] += off[c];
                lst = (int32_t*)malloc(sizeof(int32_t) * (size_t)(off[ncol] > 0 ? off[ncol] : 1));
                cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncol);
                memcpy(cur, off, sizeof(int64_t) * (size_t)ncol);
            }
            for (int64_t t = 0; t < ntri; ++t) {
                double m = marg[t];
                if (m < 0.0 || m > 1e29) continue;
                const double* T = tri + 12 * t;
                double x0 = dmin(dmin(T[0], T[3]), T[6]) - m, x1 = dmax(dmax(T[0], T[3]), T[6]) + m;
                double y0 = dmin(dmin(T[1], T[4]), T[7]) - m, y1 = dmax(dmax(T[1], T[4]), T[7]) + m;
                double fi0 = dmax(floor((x0 - org[0]) / s) - 1.0, 0.0);
                double fi1 = dmin(ceil((x1 - org[0]) / s) + 1.0, nx - 1.0);
                double fj0 = dmax(floor((y0 - org[1]) / s) - 1.0, 0.0);
                double fj1 = dmin(ceil((y1 - org[1]) / s) + 1.0, ny - 1.0);
                if (!(fi0 <= fi1) || !(fj0 <= fj1)) continue;
                int i0 = (int)fi0, i1 = (int)fi1, j0 = (int)fj0, j1 = (int)fj1;
                for (int j = j0; j <= j1; ++j) {
                    if (coly[j] < y0 || coly[j] > y1) continue;
                    for (int i = i0; i <= i1; ++i) {
                        if (colx[i] < x0 || colx[i] > x1) continue;
                        int64_t c = (int64_t)j * nx + i;
                        if (pass == 0) off[c + 1]++;
                        else lst[cur[c]++] = (int32_t)t;
                    }
                }
            }
            free(cur);
        }
        free(marg);
        free(colx);
        free(coly);
    }

    int64_t nfluid = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : nfluid)
    for (int64_t c = 0; c < ncol; ++c) {
        int i = (int)(c % nx), j = (int)(c / nx);
        for (int k = 0; k < nz; ++k) {
            double p[3], e[3];
            point_ray(bb, org, s, i, j, k, p, e);
            int count = 0;
            if (culled) {
                for (int64_t q = off[c]; q < off[c + 1]; ++q)
                    count += ray_hits(p[0], p[1], p[2], e[0], e[1], e[2], tri + 12 * (int64_t)lst[q]);
                for (int64_t q = 0; q < nglob; ++q)
                    count += ray_hits(p[0], p[1], p[2], e[0], e[1], e[2], tri + 12 * (int64_t)glob[q]);
            } else {
                for (int64_t t = 0; t < ntri; ++t)
                    count += ray_hits(p[0], p[1], p[2], e[0], e[1], e[2], tri + 12 * t);
            }
            uint8_t v = (count % 2 == 1) ? 1 : 0;
            mask[((int64_t)k * ny + j) * nx + i] = v;
            nfluid += v;
        }
    }
    free(off);
    free(lst);
    free(glob);
    return nfluid;
}

int64_t oracle_find_boundary(const uint8_t* mask, const int* dims, int Q, uint8_t* out) {
    const int nx = dims[0], ny = dims[1], nz = dims[2];
    int64_t nb = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int64_t n = ((int64_t)k * ny + j) * nx + i;
                out[n] = 0;
                if (!mask[n]) continue;
                int b = 0;
                for (int q = 0; q < Q && !b; ++q) {
                    const int* c = cvec(Q, q);
                    int a = i + c[0], bb = j + c[1], cc = k + c[2];
                    if (a >= 0 && a < nx && bb >= 0 && bb < ny && cc >= 0 && cc < nz) {
                        if (!mask[((int64_t)cc * ny + bb) * nx + a]) b = 1;
                    } else {
                        b = 1;
                    }
                }
                out[n] = (uint8_t)b;
                nb += b;
            }
    return nb;
}

/* ------------------------------------------------------------------------ */
/* solver */

struct oracle_sim {
    int Q, mode, nx, ny, nz;
    int64_t npts, nact, nnw, nwall;
    double org[3], spacing, tau;
    int64_t* pt;       /* active -> lattice point */
    uint8_t* cls;      /* active -> class */
    int32_t* nbr;      /* active*Q -> active index of x + c_q, or -1 */
    double *f, *fnew, *feq, *rho, *u;
    double* pulled;    /* physics mode: the pull's output, swapped with f after each step */
    double* prof;      /* active -> inlet profile factor */
    int64_t *nw, *wall;  /* active indices */
    double *nw_n, *wall_n, *wss, *acc, *accm, *osi, *tawss;
    oracle_bc bc[16];
    int nbc;
    int regularized;   /* physics mode: regularized collision instead of BGK */
    float* wq;         /* physics mode: wall distance per (active, arriving q), or NULL (half-way) */
    double* amp;
    int64_t namp, step;
    double C, tawss_div;
};

static int face_axis(int face) { return face / 2; }
static int face_sigma(int face) { return (face % 2 == 0) ? 1 : -1; }

static double profile_factor(const oracle_bc* b, const double* xyz) {
    if (b->profile == 0) return 1.0;
    int a = face_axis(b->face);
    int t1 = a == 0 ? 1 : 0;
    int t2 = a == 2 ? 1 : 2;
    double d1 = xyz[t1] - b->c1, d2 = xyz[t2] - b->c2;
    double p = 1.0 - (d1 * d1 + d2 * d2) / (b->R * b->R);
    return p > 0.0 ? p : 0.0;
}

oracle_sim* oracle_sim_create(int Q, int mode, const int* dims, const uint8_t* cls, const double* org,
                              double spacing, double tau, const oracle_bc* bc, int nbc) {
    if ((Q != 19 && Q != 27) || nbc < 0 || nbc > 16) return NULL;
    oracle_sim* s = (oracle_sim*)calloc(1, sizeof(oracle_sim));
    s->Q = Q; s->mode = mode;
    s->nx = dims[0]; s->ny = dims[1]; s->nz = dims[2];
    s->npts = (int64_t)s->nx * s->ny * s->nz;
    memcpy(s->org, org, sizeof(double) * 3);
    s->spacing = spacing; s->tau = tau;
    s->nbc = nbc;
    if (nbc) memcpy(s->bc, bc, sizeof(oracle_bc) * (size_t)nbc);
    int32_t* aof = (int32_t*)malloc(sizeof(int32_t) * (size_t)s->npts);
    int64_t na = 0;
    for (int64_t n = 0; n < s->npts; ++n) aof[n] = cls[n] ? (int32_t)(na++) : -1;
    s->nact = na;
    s->pt = (int64_t*)malloc(sizeof(int64_t) * (size_t)(na + 1));
    s->cls = (uint8_t*)malloc((size_t)(na + 1));
    s->nbr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(na * Q + 1));
    s->f = (double*)calloc((size_t)(na * Q + 1), sizeof(double));
    s->fnew = (double*)calloc((size_t)(na * Q + 1), sizeof(double));
    s->feq = (double*)calloc((size_t)(na * Q + 1), sizeof(double));
    s->rho = (double*)calloc((size_t)(na + 1), sizeof(double));
    s->u = (double*)calloc((size_t)(3 * na + 1), sizeof(double));
    s->prof = (double*)calloc((size_t)(na + 1), sizeof(double));
    for (int64_t n = 0, a = 0; n < s->npts; ++n) {
        if (aof[n] < 0) continue;
        s->pt[a] = n;
        s->cls[a] = cls[n];
        a++;
    }
    for (int64_t a = 0; a < na; ++a) {
        int64_t n = s->pt[a];
        int i = (int)(n % s->nx), j = (int)((n / s->nx) % s->ny), k = (int)(n / ((int64_t)s->nx * s->ny));
        for (int q = 0; q < Q; ++q) {
            const int* c = cvec(Q, q);
            int ii = i + c[0], jj = j + c[1], kk = k + c[2];
            int32_t v = -1;
            if (ii >= 0 && ii < s->nx && jj >= 0 && jj < s->ny && kk >= 0 && kk < s->nz)
                v = aof[((int64_t)kk * s->ny + jj) * s->nx + ii];
            s->nbr[a * Q + q] = v;
        }
        /* Node::Initialize (Node.cpp:30-37): f = w, fnew = 0 */
        for (int q = 0; q < Q; ++q) s->f[a * Q + q] = weight(Q, q);
        if (s->cls[a] >= 3 && s->cls[a] - 3 < nbc) {
            double xyz[3] = {org[0] + i * spacing, org[1] + j * spacing, org[2] + k * spacing};
            s->prof[a] = profile_factor(&s->bc[s->cls[a] - 3], xyz);
        }
    }
    /* next-to-wall: fluid nodes that are a lattice neighbour of a wall node
     * (Subdomain.cpp:201-218); walls listed in increasing index */
    uint8_t* isnw = (uint8_t*)calloc((size_t)(na + 1), 1);
    int64_t nwall = 0;
    for (int64_t a = 0; a < na; ++a) {
        if (s->cls[a] != 2) continue;
        nwall++;
        for (int q = 0; q < Q; ++q) {
            int32_t b = s->nbr[a * Q + q];
            if (b >= 0 && s->cls[b] == 1) isnw[b] = 1;
        }
    }
    int64_t nnw = 0;
    for (int64_t a = 0; a < na; ++a) nnw += isnw[a];
    s->nnw = nnw; s->nwall = nwall;
    s->nw = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nnw + 1));
    s->wall = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nwall + 1));
    for (int64_t a = 0, p = 0, w = 0; a < na; ++a) {
        if (isnw[a]) s->nw[p++] = a;
        if (s->cls[a] == 2) s->wall[w++] = a;
    }
    free(isnw);
    s->nw_n = (double*)calloc((size_t)(3 * nnw + 1), sizeof(double));
    s->wall_n = (double*)calloc((size_t)(3 * nwall + 1), sizeof(double));
    s->wss = (double*)calloc((size_t)(nnw + 1), sizeof(double));
    s->acc = (double*)calloc((size_t)(3 * nnw + 1), sizeof(double));
    s->accm = (double*)calloc((size_t)(nnw + 1), sizeof(double));
    s->osi = (double*)calloc((size_t)(nnw + 1), sizeof(double));
    s->tawss = (double*)calloc((size_t)(nnw + 1), sizeof(double));
    s->amp = (double*)malloc(sizeof(double));
    s->amp[0] = 0.0; s->namp = 1;
    s->C = 1.0; s->tawss_div = 0.9;
    free(aof);
    return s;
}

void oracle_sim_destroy(oracle_sim* s) {
    if (!s) return;
    free(s->pt); free(s->cls); free(s->nbr); free(s->f); free(s->fnew); free(s->feq);
    free(s->rho); free(s->u); free(s->prof); free(s->nw); free(s->wall); free(s->nw_n);
    free(s->wall_n); free(s->wss); free(s->acc); free(s->accm); free(s->osi); free(s->tawss);
    free(s->amp); free(s->wq); free(s->pulled); free(s);
}

void oracle_sim_set_amplitude(oracle_sim* s, const double* amp, int64_t n) {
    if (n < 1) return;
    free(s->amp);
    s->amp = (double*)malloc(sizeof(double) * (size_t)n);
    memcpy(s->amp, amp, sizeof(double) * (size_t)n);
    s->namp = n;
}

void oracle_sim_set_wss(oracle_sim* s, double C, double tawss_div) {
    s->C = C;
    s->tawss_div = tawss_div;
}

/* calculateBoundaryNormals (Subdomain.cpp:224-370) for one point. */
static void surface_normal(const double* tri, int64_t ntri, double x, double y, double z, double* out) {
    double n0 = 0.0, n1 = 0.0, n2 = 0.0;
    for (int64_t t = 0; t < ntri; ++t) {
        const double* T = tri + 12 * t;
        double ux = T[3] - T[0], uy = T[4] - T[1], uz = T[5] - T[2];
        double vx = T[6] - T[0], vy = T[7] - T[1], vz = T[8] - T[2];
        double nx = uy * vz - uz * vy;
        double ny = uz * vx - ux * vz;
        double nz = ux * vy - uy * vx;
        double norm = sqrt(nx * nx + ny * ny + nz * nz);
        if (norm > 0) { nx /= norm; ny /= norm; nz /= norm; }
        double area = 0.5 * norm;
        double cx = (T[0] + T[3] + T[6]) / 3.0;
        double cy = (T[1] + T[4] + T[7]) / 3.0;
        double cz = (T[2] + T[5] + T[8]) / 3.0;
        double distance = sqrt(pow(x - cx, 2) + pow(y - cy, 2) + pow(z - cz, 2));
        double w = area / (distance * distance);
        n0 += nx * w;
        n1 += ny * w;
        n2 += nz * w;
    }
    double norm = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    if (norm > 0) { n0 /= norm; n1 /= norm; n2 /= norm; }
    out[0] = n0; out[1] = n1; out[2] = n2;
}

void oracle_sim_compute_normals(oracle_sim* s, const double* tri, int64_t ntri, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int64_t tot = s->nwall + s->nnw;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t r = 0; r < tot; ++r) {
        int64_t a = r < s->nwall ? s->wall[r] : s->nw[r - s->nwall];
        double* out = r < s->nwall ? s->wall_n + 3 * r : s->nw_n + 3 * (r - s->nwall);
        int64_t n = s->pt[a];
        int i = (int)(n % s->nx), j = (int)((n / s->nx) % s->ny), k = (int)(n / ((int64_t)s->nx * s->ny));
        double x = s->org[0] + i * s->spacing, y = s->org[1] + j * s->spacing, z = s->org[2] + k * s->spacing;
        surface_normal(tri, ntri, x, y, z, out);
    }
}

/* Collision (Simulation.cpp:43-208: moments :52-175, equilibrium :183-197,
 * relaxation :201-205) for one node; f, fnew, feq point at its Q values. */
static void collide_node(int Q, double tau, const double* f, double* fnew, double* feq, double* rho_out,
                         double* u_out) {
    double density = 0.0;
    for (int q = 0; q < Q; ++q) density += f[q];
    double ux, uy, uz;
    if (Q == 19) {
        ux = ((f[0] + f[6] + f[7] + f[8] + f[9]) - (f[1] + f[10] + f[11] + f[12] + f[13])) / density;
        uy = ((f[2] + f[6] + f[10] + f[14] + f[15]) - (f[3] + f[7] + f[11] + f[16] + f[17])) / density;
        uz = ((f[4] + f[8] + f[12] + f[14] + f[16]) - (f[5] + f[9] + f[13] + f[15] + f[17])) / density;
    } else {
        ux = ((f[1] + f[7] + f[8] + f[11] + f[13] + f[19] + f[21] + f[23] + f[25]) -
              (f[2] + f[9] + f[10] + f[12] + f[14] + f[20] + f[22] + f[24] + f[26])) / density;
        uy = ((f[3] + f[7] + f[9] + f[15] + f[16] + f[19] + f[21] + f[24] + f[26]) -
              (f[4] + f[8] + f[10] + f[17] + f[18] + f[20] + f[22] + f[23] + f[25])) / density;
        uz = ((f[5] + f[11] + f[12] + f[15] + f[17] + f[19] + f[22] + f[23] + f[26]) -
              (f[6] + f[13] + f[14] + f[16] + f[18] + f[20] + f[21] + f[24] + f[25])) / density;
    }
    for (int q = 0; q < Q; ++q) {
        const int* c = cvec(Q, q);
        double du = ux * c[0] + uy * c[1] + uz * c[2];
        double u_sqr = ux * ux + uy * uy + uz * uz;
        feq[q] = weight(Q, q) * density * (1.0 + 3.0 * du + 4.5 * du * du - 1.5 * u_sqr);
    }
    for (int q = 0; q < Q; ++q) fnew[q] = f[q] + (1.0 / tau) * (feq[q] - f[q]);
    *rho_out = density;
    u_out[0] = ux; u_out[1] = uy; u_out[2] = uz;
}

/* Boundary::ApplyBc, D3Q19 (Boundary.cpp:129-157). */
static void ref_inlet_q19(double* m, double vel) {
    double u0 = vel, u1 = 0.0, u2 = 0.0;
    double rhoN = (m[2] + m[3] + m[4] + m[5] + m[14] + m[15] + m[16] + m[17] + m[18] +
                   2 * (m[1] + m[10] + m[11] + m[12] + m[13])) / (1 - u0);
    double Ny = (1.0 / 2) * (m[2] + m[14] + m[15] - m[3] - m[16] - m[17]) - (1.0 / 3) * (rhoN * u1);
    double Nz = (1.0 / 2) * (m[4] + m[16] + m[14] - m[5] - m[15] - m[17]) - (1.0 / 3) * (rhoN * u2);
    m[0] = m[1] + (1 / 3.0) * rhoN * u0;
    m[7] = m[10] + (1 / 6.0) * rhoN * (u0 - u1) + Ny;
    m[6] = m[11] + (1 / 6.0) * rhoN * (u0 + u1) - Ny;
    m[8] = m[13] + (1 / 6.0) * rhoN * (u0 + u2) - Nz;
    m[9] = m[12] + (1 / 6.0) * rhoN * (u0 - u2) + Nz;
}

/* ApplyOutletBc, outlet 1 (y-max face, Simulation.cpp:642-695). */
static void ref_outlet_ymax_q19(double* m) {
    double rho = 1.0, vx = 0.0, vz = 0.0;
    double vy = -1 + (1.0 / rho) * (m[0] + m[1] + m[4] + m[5] + m[8] + m[9] + m[12] + m[13] + m[18] +
                                    2.0 * (m[2] + m[6] + m[10] + m[14] + m[15]));
    double Nyx = 0.5 * (m[0] + m[8] + m[9] - (m[1] + m[12] + m[13])) - (1.0 / 3.0) * rho * vx;
    double Nyz = 0.5 * (m[4] + m[8] + m[12] - (m[5] + m[9] + m[13])) - (1.0 / 3.0) * rho * vz;
    m[3] = m[2] - (1.0 / 3.0) * rho * vy;
    m[11] = m[6] + (1.0 / 6.0) * rho * (-vx - vy) + Nyx;
    m[7] = m[10] + (1.0 / 6.0) * rho * (vx - vy) - Nyx;
    m[17] = m[14] + (1.0 / 6.0) * rho * (-vy - vz) + Nyz;
    m[16] = m[15] + (1.0 / 6.0) * rho * (-vy + vz) - Nyz;
}

/* ApplyOutletBc, outlets 2 and 3 (z-min face, Simulation.cpp:710-836). */
static void ref_outlet_zmin_q19(double* m) {
    double rho = 1.0, vx = 0.0, vy = 0.0;
    double vz = 1 - (1.0 / rho) * (m[0] + m[1] + m[2] + m[3] + m[6] + m[7] + m[10] + m[11] + m[18] +
                                   2.0 * (m[5] + m[9] + m[13] + m[15] + m[17]));
    double Nzx = 0.5 * (m[0] + m[6] + m[7] - (m[1] + m[10] + m[11])) - (1.0 / 3.0) * rho * vx;
    double Nzy = 0.5 * (m[2] + m[6] + m[10] - (m[3] + m[7] + m[11])) - (1.0 / 3.0) * rho * vy;
    m[4] = m[5] + (1.0 / 3.0) * rho * vz;
    m[8] = m[13] + (1.0 / 6.0) * rho * (vz + vx) - Nzx;
    m[12] = m[9] + (1.0 / 6.0) * rho * (vz - vx) + Nzx;
    m[14] = m[17] + (1.0 / 6.0) * rho * (vz + vy) - Nzy;
    m[16] = m[15] + (1.0 / 6.0) * rho * (vz - vy) + Nzy;
}

/* Zou-He on an arbitrary axis-aligned face (library semantics).  Unknowns
 * are the populations entering from outside (c_a == sigma); the transverse
 * correction divides by sum over unknowns of c_t^2 (2 for D3Q19, 6 for D3Q27). */
static void zou_he_generic(int Q, double* m, int face, int is_pressure, double value) {
    int a = face_axis(face), sg = face_sigma(face);
    double S0 = 0.0, Sm = 0.0;
    for (int q = 0; q < Q; ++q) {
        int ca = cvec(Q, q)[a];
        if (ca == 0) S0 += m[q];
        else if (ca == -sg) Sm += m[q];
    }
    double u[3] = {0.0, 0.0, 0.0};
    double rho;
    if (is_pressure) {
        rho = value;
        u[a] = sg * (1.0 - (S0 + 2.0 * Sm) / rho);
    } else {
        u[a] = sg * value;
        rho = (S0 + 2.0 * Sm) / (1.0 - sg * u[a]);
    }
    double M = Q == 19 ? 2.0 : 6.0;
    double N[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 3; ++t) {
        if (t == a) continue;
        double st = 0.0;
        for (int q = 0; q < Q; ++q) {
            const int* c = cvec(Q, q);
            if (c[a] == 0) st += m[q] * c[t];
        }
        N[t] = (st - (2.0 / 3.0) * rho * u[t]) / M;
    }
    for (int q = 0; q < Q; ++q) {
        const int* c = cvec(Q, q);
        if (c[a] != sg) continue;
        double cu = c[0] * u[0] + c[1] * u[1] + c[2] * u[2];
        double corr = 0.0;
        for (int t = 0; t < 3; ++t)
            if (t != a) corr += c[t] * N[t];
        m[q] = m[opp_of(Q, q)] + 6.0 * weight(Q, q) * rho * cu - corr;
    }
}

static void apply_bc(const oracle_sim* s, int64_t a, double* m, double amp) {
    const oracle_bc* b = &s->bc[s->cls[a] - 3];
    double vel = amp * s->prof[a] * b->value;
    if (s->Q == 19 && b->kind == ORC_BC_REF_INLET) { ref_inlet_q19(m, vel); return; }
    if (s->Q == 19 && b->kind == ORC_BC_REF_OUTLET_YMAX) { ref_outlet_ymax_q19(m); return; }
    if (s->Q == 19 && b->kind == ORC_BC_REF_OUTLET_ZMIN) { ref_outlet_zmin_q19(m); return; }
    switch (b->kind) {
        case ORC_BC_REF_INLET: zou_he_generic(s->Q, m, 0, 0, vel); break;
        case ORC_BC_REF_OUTLET_YMAX: zou_he_generic(s->Q, m, 3, 1, 1.0); break;
        case ORC_BC_REF_OUTLET_ZMIN: zou_he_generic(s->Q, m, 4, 1, 1.0); break;
        case ORC_BC_VELOCITY: zou_he_generic(s->Q, m, b->face, 0, vel); break;
        case ORC_BC_PRESSURE: zou_he_generic(s->Q, m, b->face, 1, b->value); break;
        default: break;
    }
}

/* ComputeWallShearStress (Simulation.cpp:880-898) for one node, reference
 * semantics: f post-boundary, feq from this step's collision, no (1-1/2tau). */
static void wss_ref(int Q, const double* f, const double* feq, const double* n, double C, double* tau_i) {
    for (int i = 0; i < 3; ++i) {
        double sum_alpha = 0.0;
        for (int al = 0; al < Q; ++al) {
            const int* c = cvec(Q, al);
            double sum_k = 0.0;
            for (int k = 0; k < 3; ++k) sum_k += c[k] * n[k] * n[i];
            double sum_j = 0.0;
            for (int j = 0; j < 3; ++j) sum_j += c[j] * n[j] * (c[i] - sum_k);
            double f_ne = f[al] - feq[al];
            sum_alpha += f_ne * sum_j;
        }
        tau_i[i] = C * sum_alpha;
    }
}

/* Regularized collision (physics mode, no reference counterpart: the
 * reference is BGK): f* = feq + (1 - 1/tau) f1, with the non-equilibrium part
 * projected on its second moment, f1_q = w_q / (2 cs^4) (c_q c_q - cs^2 I) : Pi,
 * Pi = sum_q (f_q - feq_q) c_q c_q, cs^2 = 1/3.  Written from the definition
 * (a direct sum over directions), so it checks the device kernel's analytic
 * form of Pi. */
static void regularize_node(int Q, double tau, const double* f, double* fnew, const double* feq) {
    double P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int q = 0; q < Q; ++q) {
        const int* c = cvec(Q, q);
        double fne = f[q] - feq[q];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) P[a][b] += fne * c[a] * c[b];
    }
    for (int q = 0; q < Q; ++q) {
        const int* c = cvec(Q, q);
        double qp = 0.0;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) qp += (c[a] * c[b] - (a == b ? 1.0 / 3.0 : 0.0)) * P[a][b];
        fnew[q] = feq[q] + (1.0 - 1.0 / tau) * weight(Q, q) * 4.5 * qp;
    }
}

void oracle_sim_set_collision(oracle_sim* s, int regularized) { s->regularized = regularized; }

/* Segment P0 -> P0 + d against one triangle (Moller and Trumbore 1997), in
 * the library's operation order: the fraction t in [0, 1] of the segment. */
static int seg_tri(const double* P0, const double* d, const double* T, double* t) {
    const double e1[3] = {T[3] - T[0], T[4] - T[1], T[5] - T[2]};
    const double e2[3] = {T[6] - T[0], T[7] - T[1], T[8] - T[2]};
    const double pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
    const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
    if (fabs(det) < 1e-300) return 0;
    const double inv = 1.0 / det;
    const double tv[3] = {P0[0] - T[0], P0[1] - T[1], P0[2] - T[2]};
    const double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv;
    if (u < 0.0 || u > 1.0) return 0;
    const double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
    const double v = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) * inv;
    if (v < 0.0 || u + v > 1.0) return 0;
    *t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
    return *t >= 0.0 && *t <= 1.0;
}

/* Wall distances for the interpolated bounce-back (no reference counterpart
 * in use: Geometry::CalculateWallDistances, ComplexGeometry.cpp:550-608,
 * computes such distances and never applies them; it divides by the spacing
 * rather than the link length).  For active node a and arriving population
 * q whose source x + c_i (i = opp q) is not active: the smallest fraction
 * t in [0, 1] of the link x -> x + c_i at which a triangle (file order) is
 * met; 0.5 where none is, and where the source exists. */
void oracle_sim_set_wall_distances(oracle_sim* s, const double* tri12, int64_t ntri) {
    const int Q = s->Q;
    free(s->wq);
    s->wq = NULL;
    if (ntri <= 0) return;
    int c[27 * 3];
    double w[27];
    int op[27];
    oracle_lattice(Q, c, w, op);
    s->wq = (float*)malloc(sizeof(float) * (size_t)(s->nact * Q + 1));
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t a = 0; a < s->nact; ++a) {
        const int64_t n = s->pt[a];
        const int i = (int)(n % s->nx), j = (int)((n / s->nx) % s->ny), k = (int)(n / ((int64_t)s->nx * s->ny));
        const double P0[3] = {s->org[0] + i * s->spacing, s->org[1] + j * s->spacing, s->org[2] + k * s->spacing};
        for (int q = 0; q < Q; ++q) {
            float qw = 0.5f;
            const int ci = op[q];
            if (s->nbr[a * Q + ci] < 0) {
                const double d[3] = {c[3 * ci] * s->spacing, c[3 * ci + 1] * s->spacing, c[3 * ci + 2] * s->spacing};
                const double lo[3] = {fmin(P0[0], P0[0] + d[0]), fmin(P0[1], P0[1] + d[1]), fmin(P0[2], P0[2] + d[2])};
                const double hi[3] = {fmax(P0[0], P0[0] + d[0]), fmax(P0[1], P0[1] + d[1]), fmax(P0[2], P0[2] + d[2])};
                double best = 2.0;
                for (int64_t r = 0; r < ntri; ++r) {
                    const double* T = tri12 + 12 * r;
                    if (fmax(T[0], fmax(T[3], T[6])) < lo[0] || fmin(T[0], fmin(T[3], T[6])) > hi[0] ||
                        fmax(T[1], fmax(T[4], T[7])) < lo[1] || fmin(T[1], fmin(T[4], T[7])) > hi[1] ||
                        fmax(T[2], fmax(T[5], T[8])) < lo[2] || fmin(T[2], fmin(T[5], T[8])) > hi[2])
                        continue;
                    double t;
                    if (seg_tri(P0, d, T, &t) && t < best) best = t;
                }
                if (best <= 1.0) qw = (float)best;
            }
            s->wq[a * Q + q] = qw;
        }
    }
}

void oracle_sim_get_wall_distances(const oracle_sim* s, float* q) {
    const int64_t n = s->nact * s->Q;
    for (int64_t k = 0; k < n; ++k) q[k] = s->wq ? s->wq[k] : 0.5f;
}

/* Library physics semantics: traction of the viscous stress
 * -(1 - 1/(2 tau)) sum_a f_neq c c, projected on the wall plane; f_neq from
 * the same post-boundary f (no time lag). */
static void wss_phys(int Q, const double* f, double tau, const double* n, double C, double* tau_i) {
    double fnew[27], feq[27], rho, u[3];
    collide_node(Q, tau, f, fnew, feq, &rho, u);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int al = 0; al < Q; ++al) {
        const int* c = cvec(Q, al);
        double cn = c[0] * n[0] + c[1] * n[1] + c[2] * n[2];
        double fne = f[al] - feq[al];
        for (int i = 0; i < 3; ++i) acc[i] += fne * cn * (c[i] - cn * n[i]);
    }
    double pref = -(1.0 - 0.5 / tau) * C;
    for (int i = 0; i < 3; ++i) tau_i[i] = pref * acc[i];
}

void oracle_sim_step(oracle_sim* s, int nsteps, int nthreads) {
    const int Q = s->Q;
    const int64_t na = s->nact;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (s->mode == ORC_PHYSICS && !s->pulled) s->pulled = (double*)malloc(sizeof(double) * (size_t)(na * Q + 1));
    for (int it = 0; it < nsteps; ++it) {
        double* g = s->pulled;
        double amp = s->amp[s->step % s->namp];
        /* collide */
#pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < na; ++a) {
            collide_node(Q, s->tau, s->f + a * Q, s->fnew + a * Q, s->feq + a * Q, s->rho + a, s->u + 3 * a);
            if (s->mode == ORC_PHYSICS && s->regularized)
                regularize_node(Q, s->tau, s->f + a * Q, s->fnew + a * Q, s->feq + a * Q);
        }
        /* stream */
        if (s->mode == ORC_PARITY) {
            /* push; a destination keeps its value when the link is missing or
             * the post-collision value is exactly zero (Simulation.cpp:220-224) */
#pragma omp parallel for schedule(static)
            for (int64_t b = 0; b < na; ++b)
                for (int q = 0; q < Q; ++q) {
                    int32_t src = s->nbr[b * Q + opp_of(Q, q)];
                    if (src >= 0 && s->fnew[(int64_t)src * Q + q] != 0.0)
                        s->f[b * Q + q] = s->fnew[(int64_t)src * Q + q];
                }
        } else {
            /* pull with half-way bounce-back for links from solid */
#pragma omp parallel for schedule(static)
            for (int64_t b = 0; b < na; ++b)
                for (int q = 0; q < Q; ++q) {
                    int32_t src = s->nbr[b * Q + opp_of(Q, q)];
                    double v = src >= 0 ? s->fnew[(int64_t)src * Q + q] : s->fnew[b * Q + opp_of(Q, q)];
                    if (src < 0 && s->wq) {
                        /* interpolated bounce-back (Bouzidi, Firdaouss and Lallemand 2001) */
                        const double qw = (double)s->wq[b * Q + q];
                        const int32_t behind = s->nbr[b * Q + q];
                        if (qw < 0.5) {
                            if (behind >= 0) {
                                const double A = 2.0 * qw;
                                v = A * v + (1.0 - A) * s->fnew[(int64_t)behind * Q + opp_of(Q, q)];
                            }
                        } else {
                            const double A = 1.0 / (2.0 * qw);
                            v = A * v + (1.0 - A) * s->fnew[b * Q + q];
                        }
                    }
                    g[b * Q + q] = v;
                }
            s->pulled = s->f;
            s->f = g;
        }
        /* boundary conditions: inlet / outlets (list order irrelevant: each node is independent) */
#pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < na; ++a)
            if (s->cls[a] >= 3) apply_bc(s, a, s->f + a * Q, amp);
        if (s->mode == ORC_PARITY) {
            /* ApplyWallBc (Simulation.cpp:843-863): in place, dir order */
#pragma omp parallel for schedule(static)
            for (int64_t w = 0; w < s->nwall; ++w) {
                int64_t a = s->wall[w];
                double* m = s->f + a * Q;
                for (int q = 0; q < Q; ++q)
                    if (s->nbr[a * Q + q] < 0) m[opp_of(Q, q)] = m[q];
            }
        }
        /* WSS + OSI/TAWSS */
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < s->nnw; ++p) {
            int64_t a = s->nw[p];
            double t[3];
            if (s->mode == ORC_PARITY) wss_ref(Q, s->f + a * Q, s->feq + a * Q, s->nw_n + 3 * p, s->C, t);
            else wss_phys(Q, s->f + a * Q, s->tau, s->nw_n + 3 * p, s->C, t);
            double WSS = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
            s->wss[p] = WSS;
            for (int i = 0; i < 3; ++i) s->acc[3 * p + i] += t[i];
            s->accm[p] += WSS;
            double tawss = s->accm[p] / s->tawss_div;
            double nrm = sqrt(pow(s->acc[3 * p], 2) + pow(s->acc[3 * p + 1], 2) + pow(s->acc[3 * p + 2], 2));
            s->osi[p] = 0.5 * (1.0 - (nrm / s->accm[p]));
            s->tawss[p] = tawss;
        }
        s->step++;
    }
}

int64_t oracle_sim_nactive(const oracle_sim* s) { return s->nact; }
int64_t oracle_sim_nnw(const oracle_sim* s) { return s->nnw; }

void oracle_sim_get_active(const oracle_sim* s, int64_t* pt, uint8_t* cls) {
    if (pt) memcpy(pt, s->pt, sizeof(int64_t) * (size_t)s->nact);
    if (cls) memcpy(cls, s->cls, (size_t)s->nact);
}

void oracle_sim_get_f(const oracle_sim* s, double* f, double* fnew, double* feq) {
    size_t n = sizeof(double) * (size_t)(s->nact * s->Q);
    if (f) memcpy(f, s->f, n);
    if (fnew) memcpy(fnew, s->fnew, n);
    if (feq) memcpy(feq, s->feq, n);
}

void oracle_sim_set_f(oracle_sim* s, const double* f) {
    memcpy(s->f, f, sizeof(double) * (size_t)(s->nact * s->Q));
}

void oracle_sim_get_macro(const oracle_sim* s, double* rho, double* u3) {
    if (rho) memcpy(rho, s->rho, sizeof(double) * (size_t)s->nact);
    if (u3) memcpy(u3, s->u, sizeof(double) * (size_t)(3 * s->nact));
}

void oracle_sim_get_nw(const oracle_sim* s, int64_t* pt, double* normal3, double* wss, double* acc3,
                       double* acc_mag, double* osi, double* tawss) {
    for (int64_t p = 0; p < s->nnw; ++p) {
        if (pt) pt[p] = s->pt[s->nw[p]];
    }
    size_t n = (size_t)s->nnw;
    if (normal3) memcpy(normal3, s->nw_n, sizeof(double) * 3 * n);
    if (wss) memcpy(wss, s->wss, sizeof(double) * n);
    if (acc3) memcpy(acc3, s->acc, sizeof(double) * 3 * n);
    if (acc_mag) memcpy(acc_mag, s->accm, sizeof(double) * n);
    if (osi) memcpy(osi, s->osi, sizeof(double) * n);
    if (tawss) memcpy(tawss, s->tawss, sizeof(double) * n);
}

void oracle_sim_get_wall_normals(const oracle_sim* s, int64_t* pt, double* normal3) {
    for (int64_t w = 0; w < s->nwall; ++w) {
        if (pt) pt[w] = s->pt[s->wall[w]];
    }
    if (normal3) memcpy(normal3, s->wall_n, sizeof(double) * 3 * (size_t)s->nwall);
}

void oracle_sim_conservation(const oracle_sim* s, double* mass, double* mom3, double* flux) {
    const int Q = s->Q;
    double m = 0.0, p[3] = {0.0, 0.0, 0.0};
    double fl[16] = {0};
    for (int64_t a = 0; a < s->nact; ++a) {
        const double* f = s->f + a * Q;
        double r = 0.0, j[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < Q; ++q) {
            const int* c = cvec(Q, q);
            r += f[q];
            j[0] += f[q] * c[0]; j[1] += f[q] * c[1]; j[2] += f[q] * c[2];
        }
        m += r;
        p[0] += j[0]; p[1] += j[1]; p[2] += j[2];
        if (s->cls[a] >= 3 && s->cls[a] - 3 < s->nbc) {
            int b = s->cls[a] - 3;
            int ax = s->bc[b].kind == ORC_BC_REF_INLET ? 0 :
                     s->bc[b].kind == ORC_BC_REF_OUTLET_YMAX ? 1 :
                     s->bc[b].kind == ORC_BC_REF_OUTLET_ZMIN ? 2 : face_axis(s->bc[b].face);
            fl[b] += j[ax];
        }
    }
    if (mass) *mass = m;
    if (mom3) { mom3[0] = p[0]; mom3[1] = p[1]; mom3[2] = p[2]; }
    if (flux) for (int b = 0; b < s->nbc; ++b) flux[b] = fl[b];
}
