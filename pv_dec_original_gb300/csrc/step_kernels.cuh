// Fused stream-collide step kernel (pull scheme), templated on lattice,
// storage format and semantics.  Included by step_f64.cu (FP64, compiled
// without FMA contraction so FP64 parity runs round exactly like the
// reference) and step_fast.cu (FP32 / FP16 / BF16 storage, FP32 arithmetic
// on offsets d = f - w).
//
// One launch advances the lattice by one reference step.  Populations are
// stored post-collision, structure of arrays, one plane per population over
// the active nodes only (plane q holds entry a, the a-th non-solid point in
// increasing n = (k*ny + j)*nx + i).  The source of the pull for population q
// is node a + delta[seg(a)][q], where a segment is a stretch of consecutive
// active nodes whose 18 neighbour offsets in active-index space agree (in
// practice an x-run of a row), so loads of a warp are contiguous and stores
// are exactly contiguous.  Launch k:
//   1. pulls f*_q(x - c_q) from the input planes        (Streaming, Simulation.cpp:211-237)
//   2. applies Zou-He / the wall rule on boundary nodes (Simulation.cpp:614-863)
//   3. accumulates wall shear stress on next-to-wall nodes (Simulation.cpp:880-898)
//   4. collides and writes f* to the output planes      (Collision, Simulation.cpp:43-208)
// so the step order of Iterate() (Simulation.cpp:577-586) is kept with the
// step boundary moved between 3 and 4; a prologue launch collides the initial
// state and a read-out launch stops after 2.
//
// Thread a handles the a-th active (non-solid) node in increasing n, so the
// 32 lanes of a warp sit on consecutive runs of x and every population load
// and store is coalesced.  One 64-bit word per node carries n, the node's
// missing-link mask and class, so every lane issues the same Q loads and the
// same Q stores; only boundary work (history, boundary rules, wall shear
// stress on next-to-wall nodes) diverges, and only those lanes look up their
// entry in the compact boundary list.
//
// Parity semantics for links whose source is missing: the reference's push
// leaves the destination's previous value in place; the boundary list keeps
// that previous post-boundary value in `stale`.  A pulled value that is
// exactly 0.0 is treated the same way (Simulation.cpp:220-224); on interior
// nodes, which keep no previous value, the event is flagged instead
// (FLAG_EXACT_ZERO) -- it needs a post-collision population of exactly zero.
#pragma once
#include <atomic>
#include <type_traits>

#include "lbm_internal.cuh"

namespace lbm {

constexpr int MODE_PARITY = LBM_PARITY;
constexpr int MODE_PHYSICS = LBM_PHYSICS;
constexpr int KIND_STEP = 0, KIND_PROLOGUE = 1, KIND_READOUT = 2;

// Momentum sums with the reference's explicit index lists (Simulation.cpp:66-175);
// the same lists apply to offsets because sum_q w_q c_q = 0.
template <int Q, typename R>
__device__ __forceinline__ void momentum(const R (&f)[Q], R& px, R& py, R& pz) {
    if constexpr (Q == 19) {
        px = (f[0] + f[6] + f[7] + f[8] + f[9]) - (f[1] + f[10] + f[11] + f[12] + f[13]);
        py = (f[2] + f[6] + f[10] + f[14] + f[15]) - (f[3] + f[7] + f[11] + f[16] + f[17]);
        pz = (f[4] + f[8] + f[12] + f[14] + f[16]) - (f[5] + f[9] + f[13] + f[15] + f[17]);
    } else {
        px = (f[1] + f[7] + f[8] + f[11] + f[13] + f[19] + f[21] + f[23] + f[25]) -
             (f[2] + f[9] + f[10] + f[12] + f[14] + f[20] + f[22] + f[24] + f[26]);
        py = (f[3] + f[7] + f[9] + f[15] + f[16] + f[19] + f[21] + f[24] + f[26]) -
             (f[4] + f[8] + f[10] + f[17] + f[18] + f[20] + f[22] + f[23] + f[25]);
        pz = (f[5] + f[11] + f[12] + f[15] + f[17] + f[19] + f[22] + f[23] + f[26]) -
             (f[6] + f[13] + f[14] + f[16] + f[18] + f[20] + f[21] + f[24] + f[25]);
    }
}

// Moments.  Full f (FP64): rho = sum f and u = j / rho with three divisions,
// as the reference rounds them (Simulation.cpp:52-175).  Offsets (FP32):
// r = rho - 1 = sum d, u = j / (1 + r).  `r` returns rho (full) or rho - 1.
template <int Q, typename R, bool OFF>
__device__ __forceinline__ void moments(const R (&f)[Q], R& r, R& ux, R& uy, R& uz) {
    R d = R(0);
#pragma unroll
    for (int q = 0; q < Q; ++q) d += f[q];
    R px, py, pz;
    momentum<Q, R>(f, px, py, pz);
    if constexpr (OFF) {
        const R inv = __frcp_rn(R(1) + d);
        ux = px * inv; uy = py * inv; uz = pz * inv;
    } else {
        ux = px / d; uy = py / d; uz = pz / d;
    }
    r = d;
}

// Equilibrium of direction q.  Full: w rho (1 + 3cu + 4.5(cu)^2 - 1.5u^2) in the
// reference's operation order (Simulation.cpp:183-197).  Offset:
// feq - w = w (r + rho (3cu + 4.5(cu)^2 - 1.5u^2)) with r = rho - 1.
template <int Q, int q, typename R, bool OFF>
__device__ __forceinline__ R feq_q(R r, R ux, R uy, R uz, R usqr) {
    const R du = ux * (R)Lat<Q>::cx(q) + uy * (R)Lat<Q>::cy(q) + uz * (R)Lat<Q>::cz(q);
    if constexpr (OFF) {
        return (R)Lat<Q>::w(q) * (r + (R(1) + r) * (R(3.0) * du + R(4.5) * du * du - R(1.5) * usqr));
    } else {
        return (R)Lat<Q>::w(q) * r * (R(1.0) + R(3.0) * du + R(4.5) * du * du - R(1.5) * usqr);
    }
}

template <int Q, typename R, bool OFF, int q = 0>
__device__ __forceinline__ void relax_all(R (&f)[Q], R r, R ux, R uy, R uz, R usqr, R inv_tau) {
    if constexpr (q < Q) {
        const R e = feq_q<Q, q, R, OFF>(r, ux, uy, uz, usqr);
        f[q] = f[q] + inv_tau * (e - f[q]);
        relax_all<Q, R, OFF, q + 1>(f, r, ux, uy, uz, usqr, inv_tau);
    }
}

template <int Q, typename R, bool OFF, int q = 0>
__device__ __forceinline__ void feq_all(R (&e)[Q], R r, R ux, R uy, R uz) {
    if constexpr (q < Q) {
        const R usqr = ux * ux + uy * uy + uz * uz;
        e[q] = feq_q<Q, q, R, OFF>(r, ux, uy, uz, usqr);
        feq_all<Q, R, OFF, q + 1>(e, r, ux, uy, uz);
    }
}


// ---------------------------------------------------------------------------
// FP32 arithmetic on offsets, with the lattice constants folded by hand:
// IEEE rules forbid the compiler to drop x * 0.0f or 0.0f + x, so products
// with c_q components are written as signed additions.

template <int c, typename R>
__device__ __forceinline__ R cadd(R s, R v) {
    if constexpr (c > 0) return s + v;
    else if constexpr (c < 0) return s - v;
    else return s;
}

// c_q . (x, y, z)
template <int Q, int q, typename R>
__device__ __forceinline__ R cdot(R x, R y, R z) {
    constexpr int cx = Lat<Q>::cx(q), cy = Lat<Q>::cy(q), cz = Lat<Q>::cz(q);
    if constexpr (cx != 0) {
        return cadd<cz>(cadd<cy>(cx > 0 ? x : -x, y), z);
    } else if constexpr (cy != 0) {
        return cadd<cz>(cy > 0 ? y : -y, z);
    } else if constexpr (cz != 0) {
        return cz > 0 ? z : -z;
    } else {
        return R(0);
    }
}

// Sums of a pair relaxation: the even parts (one per pair) and, per axis,
// sum c_a x the odd parts, for the closure of the collision invariants.
template <typename R>
struct PairSums {
    R sym = R(0), ax = R(0), ay = R(0), az = R(0);
};

// BGK relaxation of offsets d = f - w, direction pairs (q, opp q) sharing
// the even part of the equilibrium.  With A = 1 + r, B = r - 1.5 A u^2 and
// du = c_q . u:  feq_{q|opp} - w_q = w_q (B + 4.5 A du^2 +|- 3 A du), and
// d* = (1 - omega) d + omega (feq - w).  The rest population is left to
// the caller (close_invariants).
template <int Q, int q = 0>
__device__ __forceinline__ void relax_pairs(float (&f)[Q], float A, float B, float ux, float uy, float uz, float om,
                                            float om1, PairSums<float>& ps) {
    if constexpr (q < Q) {
        constexpr int o = Lat<Q>::opp(q);
        if constexpr (q != Lat<Q>::REST && q < o) {
            const float du = cdot<Q, q, float>(ux, uy, uz);
            const float ow = om * (float)Lat<Q>::w(q);
            const float t = A * du;
            const float sym = ow * ((4.5f * t) * du + B);
            const float anti = (3.0f * ow) * t;
            f[q] = om1 * f[q] + (sym + anti);
            f[o] = om1 * f[o] + (sym - anti);
            ps.sym += sym;
            ps.ax = cadd<Lat<Q>::cx(q)>(ps.ax, anti);
            ps.ay = cadd<Lat<Q>::cy(q)>(ps.ay, anti);
            ps.az = cadd<Lat<Q>::cz(q)>(ps.az, anti);
        }
        relax_pairs<Q, q + 1>(f, A, B, ux, uy, uz, om, om1, ps);
    }
}

// Closure of the collision invariants in FP32 arithmetic.  The collision
// conserves mass and momentum only through identities of the lattice
// weights (sum w = 1, sum w c c = I/3); products with the FP32-rounded
// weights break them by the same relative amount at every node and step, a
// coherent bias that accumulates (an FP32 bifurcation run drifted in mass
// against FP64 by ~5e-7 in 1000 steps, its velocity by 7e-6 -- 2.8e-5 on
// D3Q27 -- and by 1.7e-4 over 12,000 steps).  Instead of its own
// equilibrium the rest population takes the mass the pairs leave, and each
// axis pair (+a, -a) takes half the momentum defect.  With every pair
// member post-collision = keep pre + (sym +- anti):
//   sum post   = keep r + 2 sum sym + rest part        := r
//   sum c post = keep j + 2 sum c anti + 2 h (per axis) := j
// hold exactly in real arithmetic on the computed terms, so only the
// rounding of the individual results, random from node to node, remains.
// keep (the coefficient of the pre-collision values: 1 - omega for BGK, 0
// for the regularized collision) and 1 - keep must both be exact floats:
// 1 - omega is exact for 1/2 <= omega <= 2 (Sterbenz), i.e. 1/2 <= tau <= 2.
// Axis pairs: D3Q19 (0, 1) (2, 3) (4, 5); D3Q27 (1, 2) (3, 4) (5, 6).
template <int Q>
__device__ __forceinline__ void close_invariants(float (&f)[Q], const PairSums<float>& ps, float keep, float r,
                                                 float jx, float jy, float jz) {
    constexpr int XP = Q == 19 ? 0 : 1, YP = Q == 19 ? 2 : 3, ZP = Q == 19 ? 4 : 5;
    constexpr int RS = Lat<Q>::REST;
    const float give = 1.0f - keep;  // exact
    f[RS] = keep * f[RS] + (give * r - 2.0f * ps.sym);
    const float hx = fmaf(0.5f * give, jx, -ps.ax);
    const float hy = fmaf(0.5f * give, jy, -ps.ay);
    const float hz = fmaf(0.5f * give, jz, -ps.az);
    f[XP] += hx; f[Lat<Q>::opp(XP)] -= hx;
    f[YP] += hy; f[Lat<Q>::opp(YP)] -= hy;
    f[ZP] += hz; f[Lat<Q>::opp(ZP)] -= hz;
}

// Second moments sum_q d_q c_qa c_qb (xx, yy, zz, xy, xz, yz) from the
// pair sums d_q + d_opp(q): c c^T is even in c.
template <int Q, int q = 0, typename R>
__device__ __forceinline__ void second_moments(const R (&d)[Q], R (&m)[6]) {
    if constexpr (q < Q) {
        constexpr int o = Lat<Q>::opp(q);
        if constexpr (q < o) {
            constexpr int cx = Lat<Q>::cx(q), cy = Lat<Q>::cy(q), cz = Lat<Q>::cz(q);
            const R p = d[q] + d[o];
            m[0] = cadd<cx * cx>(m[0], p);
            m[1] = cadd<cy * cy>(m[1], p);
            m[2] = cadd<cz * cz>(m[2], p);
            m[3] = cadd<cx * cy>(m[3], p);
            m[4] = cadd<cx * cz>(m[4], p);
            m[5] = cadd<cy * cz>(m[5], p);
        }
        second_moments<Q, q + 1, R>(d, m);
    }
}

// Regularized collision (physics mode): the non-equilibrium part is replaced
// by its projection on the second moment,
//   f*_q = feq_q + (1 - omega) w_q 4.5 (c_q.Pi.c_q - tr Pi / 3),
//   Pi = sum_q (f_q - feq_q) c_q c_q = M - r/3 I - A u u,
// with M the second moment of the stored values (offsets d = f - w, or full
// f) and, as in relax_pairs, A = 1 + r and B = r - 1.5 A u^2 for offsets
// (A = rho for full f: both give feq - base = w (B + 4.5 A du^2 +|- 3 A du)).
// Filtering the higher moments keeps flows stable at relaxation times near
// 1/2 where BGK diverges.  kreg = 4.5 (1 - omega).
template <int Q, typename R, int q = 0>
__device__ __forceinline__ void relax_reg_pairs(R (&f)[Q], const R (&P)[6], R T3, R A, R B, R ux, R uy, R uz,
                                                R kreg, PairSums<R>& ps) {
    if constexpr (q < Q) {
        constexpr int o = Lat<Q>::opp(q);
        constexpr int cx = Lat<Q>::cx(q), cy = Lat<Q>::cy(q), cz = Lat<Q>::cz(q);
        if constexpr (q == Lat<Q>::REST) {
            f[q] = (R)Lat<Q>::w(q) * (B - kreg * T3);
        } else if constexpr (q < o) {
            // c.Pi.c with c components in {0, +-1}
            R cpc = R(0);
            cpc = cx != 0 ? cpc + P[0] : cpc;
            cpc = cy != 0 ? cpc + P[1] : cpc;
            cpc = cz != 0 ? cpc + P[2] : cpc;
            if constexpr (cx * cy != 0) cpc = cadd<cx * cy>(cadd<cx * cy>(cpc, P[3]), P[3]);
            if constexpr (cx * cz != 0) cpc = cadd<cx * cz>(cadd<cx * cz>(cpc, P[4]), P[4]);
            if constexpr (cy * cz != 0) cpc = cadd<cy * cz>(cadd<cy * cz>(cpc, P[5]), P[5]);
            const R du = cdot<Q, q, R>(ux, uy, uz);
            const R w = (R)Lat<Q>::w(q);
            const R t = A * du;
            const R e = w * ((R(4.5) * t) * du + B + kreg * (cpc - T3));
            const R anti = (R(3.0) * w) * t;
            f[q] = e + anti;
            f[o] = e - anti;
            ps.sym += e;
            ps.ax = cadd<cx>(ps.ax, anti);
            ps.ay = cadd<cy>(ps.ay, anti);
            ps.az = cadd<cz>(ps.az, anti);
        }
        relax_reg_pairs<Q, R, q + 1>(f, P, T3, A, B, ux, uy, uz, kreg, ps);
    }
}

template <int Q, typename R>
__device__ __forceinline__ void relax_regularized(R (&f)[Q], R r, R A, R ux, R uy, R uz, R om, PairSums<R>& ps) {
    R m[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
    second_moments<Q, 0, R>(f, m);
    const R r3 = r * (R(1) / R(3));
    const R P[6] = {m[0] - (r3 + A * ux * ux), m[1] - (r3 + A * uy * uy), m[2] - (r3 + A * uz * uz),
                    m[3] - A * ux * uy,        m[4] - A * ux * uz,        m[5] - A * uy * uz};
    const R T3 = (P[0] + P[1] + P[2]) * (R(1) / R(3));
    const R B = r - R(1.5) * A * (ux * ux + uy * uy + uz * uz);
    relax_reg_pairs<Q, R>(f, P, T3, A, B, ux, uy, uz, R(4.5) * (R(1) - om), ps);
}

// Wall shear stress from the non-equilibrium stress tensor
//   Pi = sum_q (f_q - feq_q) c_q c_q^T,
// using sum_q (feq_q - w_q) c_q c_q^T = r/3 I + (1 + r) u u^T (exact for the
// second-order equilibrium on D3Q19 and D3Q27): tau = C (Pi n - (n.Pi n) n),
// the per-direction sum of Simulation.cpp:880-898 regrouped.  (r, u) are the
// moments the equilibrium is taken at.
__device__ __forceinline__ void wss_from_moments(const float (&m)[6], float r, float ux, float uy, float uz,
                                                 const float n[3], float C, float t[3]) {
    const float A = 1.0f + r, r3 = r * (1.0f / 3.0f);
    const float Axx = m[0] - (r3 + A * ux * ux), Ayy = m[1] - (r3 + A * uy * uy), Azz = m[2] - (r3 + A * uz * uz);
    const float Axy = m[3] - A * ux * uy, Axz = m[4] - A * ux * uz, Ayz = m[5] - A * uy * uz;
    const float px = Axx * n[0] + Axy * n[1] + Axz * n[2];
    const float py = Axy * n[0] + Ayy * n[1] + Ayz * n[2];
    const float pz = Axz * n[0] + Ayz * n[1] + Azz * n[2];
    const float nn = px * n[0] + py * n[1] + pz * n[2];
    t[0] = C * (px - nn * n[0]);
    t[1] = C * (py - nn * n[1]);
    t[2] = C * (pz - nn * n[2]);
}

template <int Q>
__device__ __forceinline__ void wss_stress(const float (&d)[Q], float r, float ux, float uy, float uz,
                                           const float n[3], float C, float t[3]) {
    float m[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    second_moments<Q>(d, m);
    wss_from_moments(m, r, ux, uy, uz, n, C, t);
}

// ---------------------------------------------------------------------------
// Scaled formats (FP16, BF16): arithmetic on the storage units g = d / unit_q.

template <int Q, typename S>
__device__ __forceinline__ void units_to_offsets(float (&g)[Q]) {
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] *= Store<S>::template unit<Q>(q);
}

template <int Q, typename S>
__device__ __forceinline__ void offsets_to_units(float (&g)[Q]) {
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] *= 1.0f / Store<S>::template unit<Q>(q);
}

// r = rho - 1 = sum unit_q g_q and u = (sum unit_q c_q g_q) / (1 + r).
template <int Q, typename S>
__device__ __forceinline__ void moments_units(const float (&g)[Q], float& r, float& ux, float& uy, float& uz) {
    float d = 0.f, px = 0.f, py = 0.f, pz = 0.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float u = Store<S>::template unit<Q>(q);
        d = fmaf(u, g[q], d);
        if (Lat<Q>::cx(q) != 0) px = fmaf((float)Lat<Q>::cx(q) * u, g[q], px);
        if (Lat<Q>::cy(q) != 0) py = fmaf((float)Lat<Q>::cy(q) * u, g[q], py);
        if (Lat<Q>::cz(q) != 0) pz = fmaf((float)Lat<Q>::cz(q) * u, g[q], pz);
    }
    const float inv = __frcp_rn(1.0f + d);
    ux = px * inv; uy = py * inv; uz = pz * inv;
    r = d;
}

// Second moments sum_q unit_q g_q c_qa c_qb from the pair sums.
template <int Q, typename S, int q = 0>
__device__ __forceinline__ void second_moments_units(const float (&g)[Q], float (&m)[6]) {
    if constexpr (q < Q) {
        constexpr int o = Lat<Q>::opp(q);
        if constexpr (q < o) {
            constexpr int cx = Lat<Q>::cx(q), cy = Lat<Q>::cy(q), cz = Lat<Q>::cz(q);
            constexpr float u = Store<S>::template unit<Q>(q);
            const float p = g[q] + g[o];
            if constexpr (cx * cx != 0) m[0] = fmaf(u, p, m[0]);
            if constexpr (cy * cy != 0) m[1] = fmaf(u, p, m[1]);
            if constexpr (cz * cz != 0) m[2] = fmaf(u, p, m[2]);
            if constexpr (cx * cy != 0) m[3] = fmaf((float)(cx * cy) * u, p, m[3]);
            if constexpr (cx * cz != 0) m[4] = fmaf((float)(cx * cz) * u, p, m[4]);
            if constexpr (cy * cz != 0) m[5] = fmaf((float)(cy * cz) * u, p, m[5]);
        }
        second_moments_units<Q, S, q + 1>(g, m);
    }
}

// BGK relaxation in storage units, pairs (q, opp q): with K = omega geq,
// g* = (1 - omega) g + K (B + 4.5 A du^2 +|- 3 A du)  -- relax_pairs with the
// per-direction weight gone (geq is the same for every q).
template <int Q, int q = 0>
__device__ __forceinline__ void relax_pairs_units(float (&g)[Q], float A, float B, float ux, float uy, float uz,
                                                  float K, float K3, float om1) {
    if constexpr (q < Q) {
        constexpr int o = Lat<Q>::opp(q);
        if constexpr (q == Lat<Q>::REST) {
            g[q] = om1 * g[q] + K * B;
        } else if constexpr (q < o) {
            const float du = cdot<Q, q, float>(ux, uy, uz);
            const float t = A * du;
            const float sym = K * ((4.5f * t) * du + B);
            const float anti = K3 * t;
            g[q] = om1 * g[q] + (sym + anti);
            g[o] = om1 * g[o] + (sym - anti);
        }
        relax_pairs_units<Q, q + 1>(g, A, B, ux, uy, uz, K, K3, om1);
    }
}

// ---------------------------------------------------------------------------
// Boundary formulas.

// Boundary::ApplyBc, D3Q19 x-min velocity inlet (Boundary.cpp:129-157), full f.
__device__ __forceinline__ void ref_inlet_q19(double (&m)[19], double vel) {
    const double u0 = vel, u1 = 0.0, u2 = 0.0;
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

// ApplyOutletBc outlet 1, y-max face, rho = 1 (Simulation.cpp:642-695), full f.
__device__ __forceinline__ void ref_outlet_ymax_q19(double (&m)[19]) {
    const double rho = 1.0, vx = 0.0, vz = 0.0;
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

// ApplyOutletBc outlets 2 and 3, z-min face, rho = 1 (Simulation.cpp:710-836), full f.
__device__ __forceinline__ void ref_outlet_zmin_q19(double (&m)[19]) {
    const double rho = 1.0, vx = 0.0, vy = 0.0;
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

// Zou-He on any axis-aligned face.  With sigma = +1 on a min face and -1 on
// a max face, the unknowns are the populations with c_a == sigma:
//   rho (1 - sigma u_a) = S_0 + 2 S_{-sigma}
//   N_t = (sum_{c_a=0} f c_t - 2/3 rho u_t) / M      (M = 2 for D3Q19, 6 for D3Q27)
//   f_i = f_opp(i) + 6 w_i rho (c_i . u) - sum_t c_it N_t
// which reduces to the reference's formulas on its faces for both lattices
// (Boundary.cpp:87-157).  On offsets d = f - w the same lines hold with
// S_0 + 2 S_{-sigma} gaining +1 (the weights of those populations sum to 1)
// and everything else unchanged (w_i = w_opp(i), sum_{c_a=0} w c_t = 0).
// The offset form keeps rho - 1 instead of rho (a pressure rule's `value`
// is then rho - 1): S - 1 = S_0 + 2 S_{-sigma} is small, and forming S or
// rho near 1 in FP32 would round the boundary's mass flux by the same few
// 1e-8 at a node every step (an outlet's u_a = 1 - S / rho cancels down to
// the velocity), a coherent bias like the one close_invariants removes:
//   pressure:  u_a = sigma ((rho - 1) - (S - 1)) / rho
//   velocity:  rho - 1 = ((S - 1) + sigma u_a) / (1 - sigma u_a)
// with rho x formed as x + (rho - 1) x.
template <int Q, int FACE, typename R, bool OFF>
__device__ __forceinline__ void zou_he_face(R (&m)[Q], bool pressure, R value) {
    constexpr int a = FACE / 2;
    constexpr int sg = (FACE % 2 == 0) ? 1 : -1;
    R S0 = R(0), Sm = R(0);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int ca = lat_c<Q>(q, a);
        if (ca == 0) S0 += m[q];
        else if (ca == -sg) Sm += m[q];
    }
    R u[3] = {R(0), R(0), R(0)};
    R rho = R(0), rm1 = R(0);  // rho (full f) or rho - 1 (offsets)
    if constexpr (OFF) {
        const R Sp = S0 + R(2.0) * Sm;
        if (pressure) {
            rm1 = value;
            u[a] = R(sg) * (rm1 - Sp) / (R(1.0) + rm1);
        } else {
            u[a] = R(sg) * value;
            rm1 = (Sp + R(sg) * u[a]) / (R(1.0) - R(sg) * u[a]);
        }
    } else {
        const R S = S0 + R(2.0) * Sm;
        if (pressure) {
            rho = value;
            u[a] = R(sg) * (R(1.0) - S / rho);
        } else {
            u[a] = R(sg) * value;
            rho = S / (R(1.0) - R(sg) * u[a]);
        }
    }
    R N[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        if (t == a) continue;
        R st = R(0);
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (lat_c<Q>(q, a) == 0) st += m[q] * (R)lat_c<Q>(q, t);
        if constexpr (OFF) N[t] = (st - (R(2.0) / R(3.0)) * (u[t] + rm1 * u[t])) / (R)Lat<Q>::ZH_M;
        else N[t] = (st - (R(2.0) / R(3.0)) * rho * u[t]) / (R)Lat<Q>::ZH_M;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (lat_c<Q>(q, a) != sg) continue;
        const R cu = (R)Lat<Q>::cx(q) * u[0] + (R)Lat<Q>::cy(q) * u[1] + (R)Lat<Q>::cz(q) * u[2];
        R corr = R(0);
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (t != a) corr += (R)lat_c<Q>(q, t) * N[t];
        if constexpr (OFF) m[q] = m[Lat<Q>::opp(q)] + R(6.0) * (R)Lat<Q>::w(q) * (cu + rm1 * cu) - corr;
        else m[q] = m[Lat<Q>::opp(q)] + R(6.0) * (R)Lat<Q>::w(q) * rho * cu - corr;
    }
}

template <int Q, typename R, bool OFF>
__device__ __forceinline__ void zou_he(R (&m)[Q], int face, bool pressure, R value) {
    switch (face) {
        case 0: zou_he_face<Q, 0, R, OFF>(m, pressure, value); break;
        case 1: zou_he_face<Q, 1, R, OFF>(m, pressure, value); break;
        case 2: zou_he_face<Q, 2, R, OFF>(m, pressure, value); break;
        case 3: zou_he_face<Q, 3, R, OFF>(m, pressure, value); break;
        case 4: zou_he_face<Q, 4, R, OFF>(m, pressure, value); break;
        default: zou_he_face<Q, 5, R, OFF>(m, pressure, value); break;
    }
}

// The reference's literal D3Q19 formulas run where they can be bit-exact
// (FP64, full f); elsewhere the reference kinds use the equivalent face form.
template <int Q, typename R, bool OFF>
__device__ __forceinline__ void apply_bc(R (&m)[Q], const BCDev& b, double amp, double prof) {
    // FP64 keeps the reference's product (amplitude * profile); FP32 multiplies in FP32
    R vel;
    if constexpr (OFF) vel = (R)amp * (R)prof * (R)b.value;
    else vel = amp * prof * b.value;
    // the reference outlets' density as zou_he_face takes it: rho, or rho - 1 on offsets
    const R unit_rho = OFF ? R(0.0) : R(1.0);
    if constexpr (Q == 19 && !OFF) {
        if (b.kind == LBM_BC_REF_INLET) { ref_inlet_q19(m, vel); return; }
        if (b.kind == LBM_BC_REF_OUTLET_YMAX) { ref_outlet_ymax_q19(m); return; }
        if (b.kind == LBM_BC_REF_OUTLET_ZMIN) { ref_outlet_zmin_q19(m); return; }
    } else {
        if (b.kind == LBM_BC_REF_INLET) { zou_he<Q, R, OFF>(m, LBM_FACE_XMIN, false, vel); return; }
        if (b.kind == LBM_BC_REF_OUTLET_YMAX) { zou_he<Q, R, OFF>(m, LBM_FACE_YMAX, true, unit_rho); return; }
        if (b.kind == LBM_BC_REF_OUTLET_ZMIN) { zou_he<Q, R, OFF>(m, LBM_FACE_ZMIN, true, unit_rho); return; }
    }
    if (b.kind == LBM_BC_VELOCITY) zou_he<Q, R, OFF>(m, b.face, false, vel);
    else if (b.kind == LBM_BC_PRESSURE) zou_he<Q, R, OFF>(m, b.face, true, OFF ? (R)b.value_m1 : (R)b.value);
}

__device__ __forceinline__ int bc_axis(const BCDev& b) {
    return b.kind == LBM_BC_REF_INLET ? 0 : b.kind == LBM_BC_REF_OUTLET_YMAX ? 1
                                          : b.kind == LBM_BC_REF_OUTLET_ZMIN ? 2 : b.face / 2;
}

// ---------------------------------------------------------------------------
// Wall shear stress.

// Reference form (Simulation.cpp:880-898): literal loop nest, FP64.
template <int Q>
__device__ __forceinline__ void wss_reference(const double (&f)[Q], const double (&feq)[Q], const double n[3],
                                              double C, double tau_i[3]) {
    for (int i = 0; i < 3; ++i) {
        double sum_alpha = 0.0;
#pragma unroll
        for (int al = 0; al < Q; ++al) {
            const double c[3] = {(double)Lat<Q>::cx(al), (double)Lat<Q>::cy(al), (double)Lat<Q>::cz(al)};
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

// Same quantity, factored: tau_i = C sum_a f_ne (c.n)(c_i - (c.n) n_i), with
// the equilibrium of moments (r, u) evaluated inside the loop.
template <int Q, typename R, bool OFF>
__device__ __forceinline__ void wss_fast(const R (&f)[Q], R r, R ux, R uy, R uz, const R n[3], R C, R tau_i[3]) {
    const R usqr = ux * ux + uy * uy + uz * uz;
    R a0 = R(0), a1 = R(0), a2 = R(0);
#pragma unroll
    for (int al = 0; al < Q; ++al) {
        const R cx = (R)Lat<Q>::cx(al), cy = (R)Lat<Q>::cy(al), cz = (R)Lat<Q>::cz(al);
        const R du = ux * cx + uy * cy + uz * cz;
        const R e = OFF ? (R)Lat<Q>::w(al) * (r + (R(1) + r) * (R(3.0) * du + R(4.5) * du * du - R(1.5) * usqr))
                        : (R)Lat<Q>::w(al) * r * (R(1.0) + R(3.0) * du + R(4.5) * du * du - R(1.5) * usqr);
        const R cn = cx * n[0] + cy * n[1] + cz * n[2];
        const R k = (f[al] - e) * cn;
        a0 += k * (cx - cn * n[0]);
        a1 += k * (cy - cn * n[1]);
        a2 += k * (cz - cn * n[2]);
    }
    tau_i[0] = C * a0; tau_i[1] = C * a1; tau_i[2] = C * a2;
}

// Compensated accumulation in two floats (Neumaier): acc.x carries the sum,
// acc.y the rounding errors; the value is (double)acc.x + acc.y.
__device__ __forceinline__ void comp_add(float2& acc, float v) {
    const float s = acc.x + v;
    const float c = fabsf(acc.x) >= fabsf(v) ? (acc.x - s) + v : (v - s) + acc.x;
    acc.x = s;
    acc.y += c;
}

// Fold one half of the FP32 stress ring (slots half * kFoldEvery ..
// + kFoldEvery - 1, i.e. kFoldEvery consecutive steps in step order) into
// next-to-wall node nw's compensated accumulators.
template <bool CG = false>
__device__ __forceinline__ void fold_half(const StepParams& P, int64_t nw, int half) {
    const float4* __restrict__ ring = reinterpret_cast<const float4*>(P.nw_ring);
    float2 acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = P.nw_accf[k * P.nnw + nw];
#pragma unroll 4
    for (int j = 0; j < kFoldEvery; ++j) {
        const float4* src = ring + (int64_t)(half * kFoldEvery + j) * P.nnw + nw;
        const float4 v = CG ? __ldcg(src) : *src;
        comp_add(acc[0], v.x);
        comp_add(acc[1], v.y);
        comp_add(acc[2], v.z);
        comp_add(acc[3], v.w);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) P.nw_accf[k * P.nnw + nw] = acc[k];
}

// The fold blocks of a step launch (the first P.fold_blocks blocks, BT
// threads each): at a step whose index is a multiple of kFoldEvery, fold
// the half of the ring this step does not write.
// Each fold thread folds next-to-wall nodes a fold-grid apart (a step
// launch carries one fold block per kFoldNodes x block size nodes).
constexpr int kFoldNodes = 4;
__device__ __forceinline__ void fold_blocks_work(const StepParams& P, int64_t block, int bt) {
    const int64_t step = *P.step_base;
    if (step % kFoldEvery != 0) return;
    const int writing = (int)((step % kRingSlots) / kFoldEvery);
    const int64_t stride = (int64_t)(P.fold_blocks > 0 ? P.fold_blocks : gridDim.x) * bt;
    for (int64_t nw = block * bt + threadIdx.x; nw < P.nnw; nw += stride) fold_half(P, nw, 1 - writing);
}

// The same as a kernel of its own, after a step launch without fold blocks.
static __global__ void k_fold_ring(const StepParams P) { fold_blocks_work(P, blockIdx.x, blockDim.x); }

// ---------------------------------------------------------------------------
// Block reduction of the read-out sums (rho - 1, momentum, per-BC flux).

template <int BT>
__device__ __forceinline__ void block_partials(double (&v)[kPartialStride], double* __restrict__ out) {
    __shared__ double red[BT / 32][kPartialStride];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kPartialStride; ++k) {
        double x = v[k];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
        if (lane == 0) red[warp][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < kPartialStride) {
        double s = 0.0;
        for (int w = 0; w < BT / 32; ++w) s += red[w][threadIdx.x];
        out[(int64_t)blockIdx.x * kPartialStride + threadIdx.x] = s;
    }
}

template <int Q, typename R, bool OFF>
__device__ __forceinline__ double full_value(R v, int q) {
    return OFF ? Lat<Q>::w(q) + (double)v : (double)v;
}

// f* == 0.0 in the arithmetic's own representation.
template <int Q, typename R, bool OFF>
__device__ __forceinline__ bool is_exact_zero(R v, int q) {
    return OFF ? (v == -(R)Lat<Q>::w(q)) : (v == R(0));
}

// ---------------------------------------------------------------------------
// The kernel.



// Packed per-node word (built by setup.cu):
//   bits  0-30  segment id: the pull source of population q is node a + delta[seg][q]
//   bit   31    boundary-list node (needs the long path)
//   bits 32-58  missing-link mask: bit q set when x + c_q is solid / outside
//   bits 59-62  class (1 fluid, 2 wall, 3 boundary condition: its rule is sp_bc of the entry)
//   bit   63    next-to-wall node (accumulates wall shear stress)
__device__ __forceinline__ int64_t word_segment(uint64_t w) { return (int64_t)(w & 0x7fffffffull); }
__device__ __forceinline__ bool word_special(uint64_t w) { return (w >> 31) & 1ull; }
__device__ __forceinline__ uint32_t word_miss(uint64_t w) { return (uint32_t)((w >> 32) & 0x7ffffffull); }
__device__ __forceinline__ int word_class(uint64_t w) { return (int)((w >> 59) & 0xfull); }
__device__ __forceinline__ bool word_nw(uint64_t w) { return (w >> 63) & 1ull; }

// After the pull: boundary rules, wall shear stress, collision and store
// (or the read-out sums) of node a with post-stream populations g.  nr and
// slot: the next-to-wall normal and stress-ring slot (FP32 formats).
template <int Q, typename S, int MODE, int KIND, bool WIDE>
__device__ __forceinline__ void node_finish(const StepParams& P, const int64_t a, const uint64_t word,
                                            const int64_t s, const bool lng, const int c, const uint32_t miss,
                                            typename Store<S>::real (&g)[Q], const float (&nr)[3], const int slot,
                                            double (&part)[kPartialStride]) {
    using I = typename std::conditional<WIDE, int64_t, int32_t>::type;
    using R = typename Store<S>::real;
    constexpr bool OFF = Store<S>::offset;
    constexpr bool SC = Store<S>::scaled;  // g in storage units (FP16, BF16)
    S* __restrict__ fout = static_cast<S*>(P.fout);
    const bool direct = (KIND == KIND_PROLOGUE) || (KIND == KIND_READOUT && P.direct);
    constexpr bool parity_readout = (KIND == KIND_READOUT && MODE == MODE_PARITY);
    const I ai = (I)a, st = (I)P.stride;
    // f == 0 in the values g holds
    auto exact_zero = [](R v, int q) {
        if constexpr (SC) return v == -(R)Store<S>::geq;
        else return is_exact_zero<Q, R, OFF>(v, q);
    };
    // rho - 1 (or rho) and u of g
    auto mom = [](const R (&v)[Q], R& r, R& ux, R& uy, R& uz) {
        if constexpr (SC) moments_units<Q, S>(v, r, ux, uy, uz);
        else moments<Q, R, OFF>(v, r, ux, uy, uz);
    };
    int nw = -1;  // next-to-wall index: boundary-list entries below nnw
    if (lng) {
        // ---- boundary-list node: history, boundary rules
        R* __restrict__ stale = static_cast<R*>(P.stale);
        if constexpr (MODE == MODE_PARITY) {
            if (parity_readout) {
                // the boundary list keeps the exact post-boundary f of the last step
#pragma unroll
                for (int q = 0; q < Q; ++q) g[q] = stale[q * P.nsp + s];
            } else if (!direct) {
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    if (((miss >> Lat<Q>::opp(q)) & 1u) || exact_zero(g[q], q))
                        g[q] = stale[q * P.nsp + s];
            }
        }
        if (!direct && !parity_readout) {
            if (c >= CLS_BC0) {
                int32_t rule = __ldg(P.sp_bc + s);
                if (!in_bounds(rule, P.nbc, P.flags)) rule = 0;
                const BCDev& B = P.bct[rule];
                double amp = 0.0;
                const int64_t len = __ldg(P.wave_len + B.wave);
                if (len > 0) {
                    int64_t t = (*P.step_base + P.step_off) % len;
                    if (t < 0) t += len;
                    amp = __ldg(P.amp + __ldg(P.wave_off + B.wave) + t);
                }
                if constexpr (SC) units_to_offsets<Q, S>(g);
                apply_bc<Q, R, OFF>(g, B, amp, __ldg(P.sp_prof + s));
                if constexpr (SC) offsets_to_units<Q, S>(g);
            } else if (MODE == MODE_PARITY && c == CLS_WALL) {
                // ApplyWallBc: in place, direction order (Simulation.cpp:846-861)
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    if ((miss >> q) & 1u) g[Lat<Q>::opp(q)] = g[q];
            }
        }
        if constexpr (KIND == KIND_READOUT) {
            if (c >= CLS_BC0) {
                R r, ux, uy, uz;
                mom(g, r, ux, uy, uz);
                const double rho = OFF ? 1.0 + (double)r : (double)r;
                const double j[3] = {rho * ux, rho * uy, rho * uz};
                P.sp_flux[s] = j[bc_axis(P.bct[__ldg(P.sp_bc + s)])];
            }
        }
        if (s < P.nnw) nw = (int)s;
    } else if constexpr (MODE == MODE_PARITY && KIND == KIND_STEP) {
        bool zero = false;
#pragma unroll
        for (int q = 0; q < Q; ++q) zero |= exact_zero(g[q], q);
        if (zero) atomicOr(P.flags, FLAG_EXACT_ZERO);
    }

    if constexpr (KIND == KIND_READOUT) {
        R r, ux, uy, uz;
        mom(g, r, ux, uy, uz);
        const double rho = OFF ? 1.0 + (double)r : (double)r;
        part[0] = OFF ? (double)r : rho - 1.0;
        part[1] = rho * ux; part[2] = rho * uy; part[3] = rho * uz;
        if (P.out_f || P.out_rho) {
            double fd[Q];  // the full f in FP64
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                if constexpr (SC)
                    fd[q] = Lat<Q>::w(q) + (double)Store<S>::template unit<Q>(q) * (double)g[q];
                else
                    fd[q] = full_value<Q, R, OFF>(g[q], q);
            }
            if (P.out_f) {
#pragma unroll
                for (int q = 0; q < Q; ++q) P.out_f[a * Q + q] = fd[q];
            }
            if (P.out_rho) {
                // the FP64 moments of the full f (Collision's formulas), as
                // the FP64 distributions of lbm_get_distributions would give them
                double rr, vx, vy, vz;
                moments<Q, double, false>(fd, rr, vx, vy, vz);
                P.out_rho[a] = rr;
                P.out_u[3 * a] = vx; P.out_u[3 * a + 1] = vy; P.out_u[3 * a + 2] = vz;
            }
        }
    } else {
        // ---- moments of the post-boundary populations: they serve the
        // wall shear stress (physics), the next step's lagged stress
        // (parity) and the collision
        R r, ux, uy, uz;
        mom(g, r, ux, uy, uz);
        float jx = 0.f, jy = 0.f, jz = 0.f;  // momentum of g (FP32 offsets: the collision invariants)
        if constexpr (OFF && !SC) momentum<Q, float>(g, jx, jy, jz);
        R* __restrict__ prev = static_cast<R*>(P.nw_prev);
        if (KIND == KIND_STEP && nw >= 0) {
            if constexpr (!OFF) {
                // FP64: the reference's arithmetic
                double t[3];
                const double nn[3] = {P.nw_n[nw], P.nw_n[P.nnw + nw], P.nw_n[2 * P.nnw + nw]};
                if constexpr (MODE == MODE_PARITY) {
                    // equilibrium of the previous collision (time-lagged, as the reference)
                    double e[Q];
                    feq_all<Q, double, false>(e, prev[nw], prev[P.nnw + nw], prev[2 * P.nnw + nw],
                                              prev[3 * P.nnw + nw]);
                    wss_reference<Q>(g, e, nn, P.wss_C, t);
                } else {
                    wss_fast<Q, double, false>(g, r, ux, uy, uz, nn, P.wss_phys, t);
                }
                const double W = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
                P.nw_wss[nw] = W;
                P.nw_acc[nw] += t[0];
                P.nw_acc[P.nnw + nw] += t[1];
                P.nw_acc[2 * P.nnw + nw] += t[2];
                P.nw_accm[nw] += W;
            } else {
                // FP32 arithmetic end to end
                float t[4];
                float m[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if constexpr (SC) second_moments_units<Q, S>(g, m);
                else second_moments<Q>(g, m);
                if constexpr (MODE == MODE_PARITY) {
                    wss_from_moments(m, prev[nw], prev[P.nnw + nw], prev[2 * P.nnw + nw], prev[3 * P.nnw + nw], nr,
                                     P.wss_C_f, t);
                } else {
                    wss_from_moments(m, r, ux, uy, uz, nr, P.wss_phys_f, t);
                }
                // |tau| through the reciprocal square root (a few ulp; the
                // IEEE square root takes its special-case path for every
                // zero stress, as at rest)
                const float t2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
                t[3] = t2 > 0.f ? t2 * rsqrtf(t2) : 0.f;
                // this step's slot of the ring (folded kFoldEvery steps later)
                reinterpret_cast<float4*>(P.nw_ring)[(int64_t)slot * P.nnw + nw] = make_float4(t[0], t[1], t[2], t[3]);
            }
        }
        if constexpr (MODE == MODE_PARITY) {
            if (lng) {
                R* __restrict__ stale = static_cast<R*>(P.stale);
#pragma unroll
                for (int q = 0; q < Q; ++q) stale[q * P.nsp + s] = g[q];
                if (nw >= 0) {
                    // moments of this step's collision, for the next step's lagged stress
                    prev[nw] = r; prev[P.nnw + nw] = ux; prev[2 * P.nnw + nw] = uy; prev[3 * P.nnw + nw] = uz;
                }
            }
        }
        // ---- collide and store (every lane)
        if (MODE == MODE_PHYSICS && P.collision == LBM_COLLISION_REGULARIZED) {
            if constexpr (SC) {
                PairSums<float> ps;
                units_to_offsets<Q, S>(g);
                relax_regularized<Q, float>(g, r, 1.0f + r, ux, uy, uz, P.inv_tau_f, ps);
                offsets_to_units<Q, S>(g);
            } else if constexpr (OFF) {
                // FP32: the invariants closed (the regularized values replace f: keep = 0)
                PairSums<float> ps;
                relax_regularized<Q, float>(g, r, 1.0f + r, ux, uy, uz, P.inv_tau_f, ps);
                close_invariants<Q>(g, ps, 0.0f, r, jx, jy, jz);
            } else {
                PairSums<R> ps;
                relax_regularized<Q, R>(g, r, r, ux, uy, uz, (R)P.inv_tau, ps);
            }
        } else if constexpr (SC) {
            const float om = P.inv_tau_f;
            const float A = 1.0f + r;
            const float B = r - 1.5f * A * (ux * ux + uy * uy + uz * uz);
            const float K = om * Store<S>::geq;
            relax_pairs_units<Q>(g, A, B, ux, uy, uz, K, 3.0f * K, 1.0f - om);
        } else if constexpr (OFF) {
            // FP32: BGK pairs, then the invariants closed (keep = 1 - omega)
            const float om = P.inv_tau_f;
            const float om1 = 1.0f - om;
            const float A = 1.0f + r;
            const float B = r - 1.5f * A * (ux * ux + uy * uy + uz * uz);
            PairSums<float> ps;
            relax_pairs<Q>(g, A, B, ux, uy, uz, om, om1, ps);
            close_invariants<Q>(g, ps, om1, r, jx, jy, jz);
        } else {
            relax_all<Q, R, OFF>(g, r, ux, uy, uz, ux * ux + uy * uy + uz * uz, (R)P.inv_tau);
        }
        if (!(fabsf((float)r) < 1e30f)) atomicOr(P.flags, FLAG_NONFINITE);
        S* __restrict__ fout_a = fout + ai;
#pragma unroll
        for (int q = 0; q < Q; ++q) fout_a[q * st] = Store<S>::template pack<Q>(g[q], q);
    }
}

// Interpolated bounce-back (Bouzidi, Firdaouss and Lallemand 2001) for the
// missing links of node a, whose g[q] holds the half-way value f*_opp(q)(x):
//   q_w < 1/2: g[q] = 2 q_w f*_i(x) + (1 - 2 q_w) f*_i(x + c_q)
//   q_w >= 1/2: g[q] = f*_i(x) / (2 q_w) + (1 - 1/(2 q_w)) f*_q(x),  i = opp q.
// Compiled only into the kernels launched when wall distances are set
// (WALLS), so the half-way kernels carry none of it.
template <int Q, typename S, bool WIDE, bool CG = false>
__device__ __forceinline__ void interpolate_walls(const StepParams& P, int64_t a, uint64_t word, int32_t e,
                                                       uint32_t miss, typename Store<S>::real (&g)[Q]) {
    using I = typename std::conditional<WIDE, int64_t, int32_t>::type;
    using R = typename Store<S>::real;
    constexpr int DR = kDeltaRow<Q>;
    const S* __restrict__ fin_a = static_cast<const S*>(P.fin) + (I)a;
    const I st = (I)P.stride;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (q == Lat<Q>::REST || !((miss >> Lat<Q>::opp(q)) & 1u)) continue;
        const float qw = __ldg(P.sp_q + (int64_t)q * P.nsp + e);
        R A, X;
        if (qw < 0.5f) {
            if ((miss >> q) & 1u) continue;  // no fluid node at x + c_q: half-way
            A = (R)2 * (R)qw;
            const int32_t dq = __ldg(P.seg_delta + word_segment(word) * DR + Lat<Q>::opp(q));
            X = Store<S>::template load<Q, CG>(fin_a + (I)(Lat<Q>::opp(q) * st + dq), q);
        } else {
            A = (R)1 / ((R)2 * (R)qw);
            X = Store<S>::template load<Q, CG>(fin_a + (I)(q * st), q);
        }
        g[q] = A * g[q] + ((R)1 - A) * X;
    }
}

// What the pull of a node leaves for node_finish besides its populations.
struct Pulled {
    bool lng;        // boundary-list work
    int c;           // class
    uint32_t miss;   // missing-link mask
    int64_t s;       // boundary-list entry (lng)
    float nr[3];     // next-to-wall normal (FP32-arithmetic formats)
    int slot;        // stress-ring slot
};

// The pull of node a: its populations after streaming (and, with WALLS,
// interpolated bounce-back) into g, plus its boundary-list data.  CG: the
// populations are read from L2 (a persistent launch, see Store::load).
template <int Q, typename S, int MODE, int KIND, bool WIDE, bool WALLS = false, bool CG = false>
__device__ __forceinline__ void pull_node(const StepParams& P, const int64_t a, const uint64_t word,
                                          const int32_t sp_entry, typename Store<S>::real (&g)[Q], Pulled& pl) {
    using I = typename std::conditional<WIDE, int64_t, int32_t>::type;
    using R = typename Store<S>::real;
    constexpr bool OFF = Store<S>::offset;
    constexpr int DR = kDeltaRow<Q>;
    const S* __restrict__ fin = static_cast<const S*>(P.fin);
    const bool direct = (KIND == KIND_PROLOGUE) || (KIND == KIND_READOUT && P.direct);
    const uint32_t miss = word_miss(word);  // zero on interior nodes
    const int c = word_class(word);
    // Boundary-list work: in parity mode every boundary-list node (history
    // of missing links, the wall rule); in physics mode only
    // boundary-condition and next-to-wall nodes (bounce-back is folded
    // into the loads).  The list entry is fetched before the loads.
    const bool lng = MODE == MODE_PARITY ? word_special(word) : (c >= CLS_BC0 || word_nw(word));
    int64_t s = lng ? (int64_t)sp_entry : 0;
    if (lng && !in_bounds(s, P.nsp, P.flags)) s = 0;
    // FP32 formats: a next-to-wall node loads its normal now, beside the
    // populations, so the stress below waits on nothing
    float nr[3] = {0.f, 0.f, 0.f};
    int slot = 0;
    if constexpr (OFF && KIND == KIND_STEP) {
        if (lng && s < P.nnw) {
            nr[0] = __ldg(P.nw_nf + s);
            nr[1] = __ldg(P.nw_nf + P.nw_stride + s);
            nr[2] = __ldg(P.nw_nf + 2 * P.nw_stride + s);
            slot = (int)(*P.step_base % kRingSlots);
        }
    }

    // ---- stream: one load per population, issued by every lane together.
    // A link whose source is missing reads, in physics mode, the node's
    // own opposite population (half-way bounce-back); in parity mode any
    // valid address -- the previous value replaces it below.
    const I ai = (I)a, st = (I)P.stride;
    // the node's own entry of plane 0; plane q is q * stride further
    const S* __restrict__ fin_a = fin + ai;
    if (direct) {
#pragma unroll
        for (int q = 0; q < Q; ++q) g[q] = Store<S>::template load<Q, CG>(fin_a + q * st, q);
    } else {
        int32_t dl[DR];
        const int64_t seg = in_bounds(word_segment(word), P.nseg, P.flags) ? word_segment(word) : 0;
        const int4* __restrict__ drow = reinterpret_cast<const int4*>(P.seg_delta + seg * DR);
#pragma unroll
        for (int k = 0; k < DR / 4; ++k) {
            const int4 v = __ldg(drow + k);
            dl[4 * k] = v.x; dl[4 * k + 1] = v.y; dl[4 * k + 2] = v.z; dl[4 * k + 3] = v.w;
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const bool src_missing = (miss >> Lat<Q>::opp(q)) & 1u;
            I off;  // from the node's own entry of plane 0
            if (q == Lat<Q>::REST) {
                off = q * st;
            } else if (MODE == MODE_PHYSICS) {
                off = src_missing ? Lat<Q>::opp(q) * st : q * st + dl[q];
            } else {
                off = q * st + (src_missing ? 0 : dl[q]);
            }
            if (in_bounds((int64_t)ai + (int64_t)off, (int64_t)Q * P.stride, P.flags))
                g[q] = Store<S>::template load<Q, CG>(fin_a + off, q);  // w_opp(q) == w_q: same decode
            else
                g[q] = R(0);
        }
        if constexpr (MODE == MODE_PHYSICS && WALLS) {
            // interpolated bounce-back (the launcher picks this kernel when wall distances are set)
            if (miss != 0) interpolate_walls<Q, S, WIDE, CG>(P, a, word, sp_entry, miss, g);
        }
    }

    pl.lng = lng;
    pl.c = c;
    pl.miss = miss;
    pl.s = s;
    pl.nr[0] = nr[0]; pl.nr[1] = nr[1]; pl.nr[2] = nr[2];
    pl.slot = slot;
}

// One node's update: pull, boundary rules, wall shear stress, collision and
// store (or the read-out sums).
template <int Q, typename S, int MODE, int KIND, bool WIDE, bool WALLS = false, bool CG = false>
__device__ __forceinline__ void node_update(const StepParams& P, const int64_t a, const uint64_t word,
                                            const int32_t sp_entry, double (&part)[kPartialStride]) {
    typename Store<S>::real g[Q];
    Pulled pl;
    pull_node<Q, S, MODE, KIND, WIDE, WALLS, CG>(P, a, word, sp_entry, g, pl);
    node_finish<Q, S, MODE, KIND, WIDE>(P, a, word, pl.s, pl.lng, pl.c, pl.miss, g, pl.nr, pl.slot, part);
}

// Programmatic dependent launch: a step kernel is launched with
// programmatic stream serialization, so it may start while the previous
// kernel of the stream finishes.  Each block reads its read-only node data,
// then waits (pdl_wait) for the previous grid to complete and its writes to
// be visible before it reads or writes any state.  Without a preceding
// dependent launch the wait returns at once.  The next launch begins once
// every block has called pdl_trigger: at block start when the grid is
// larger than one wave of resident blocks (P.pdl_early; the next grid's
// blocks then take the SMs this grid's tail leaves), at block end otherwise
// (a grid that fits at once would have the next grid's blocks wait beside
// its running blocks: 83k-node lattices stepped 12% slower).
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// WIDE = false: population offsets q * stride + a in 32-bit arithmetic, for
// lattices with Q * stride < 2^31 (the launcher checks); WIDE = true: 64-bit.
// One thread per active node.
template <int Q, typename S, int MODE, int KIND, int BT = kStepThreads, int MINB = 1, bool WIDE = true,
          bool WALLS = false>
__global__ void __launch_bounds__(BT, MINB) step_kernel(const StepParams P) {
    double part[kPartialStride];
    if constexpr (KIND == KIND_READOUT) {
#pragma unroll
        for (int k = 0; k < kPartialStride; ++k) part[k] = 0.0;
    }
    int64_t blk = blockIdx.x;
    if constexpr (KIND == KIND_STEP) {
        if (P.pdl_early) pdl_trigger();
        if constexpr (Store<S>::offset) {
            // leading blocks: the stress ring's fold (FP32-arithmetic formats)
            if (blk < P.fold_blocks) {
                pdl_wait();
                if (blockIdx.x == 0 && threadIdx.x == 0) *P.step_next = *P.step_base + 1;
                fold_blocks_work(P, blk, BT);
                if (!P.pdl_early) pdl_trigger();
                return;
            }
            blk -= P.fold_blocks;
        }
    }
    if constexpr (KIND == KIND_STEP) {
        // blocks from both ends of the active-node order first, meeting in
        // the middle: a vessel along the slowest lattice axis has its inlet
        // and outlet planes (the slowest blocks) at the two ends, and
        // starting them first keeps them out of the launch's tail
        // (bifurcation: FP32 step -6%, FP16 -4.5%)
        const int64_t nm = (P.nact + BT - 1) / BT;
        blk = (blk & 1) ? nm - 1 - (blk >> 1) : (blk >> 1);
    }
    const int64_t a = blk * BT + threadIdx.x;
    // the node's word and its boundary-list entry (-1 for most nodes),
    // loaded side by side (read-only: before the dependency wait)
    uint64_t word = 0;
    int32_t sp_entry = -1;
    if (a < P.nact) {
        word = __ldg(P.act_word + a);
        sp_entry = __ldg(P.sp_of_act + a);
    }
    if constexpr (KIND == KIND_STEP) {
        pdl_wait();
        // block 0 is a node block when there are no fold blocks
        if (blockIdx.x == 0 && threadIdx.x == 0) *P.step_next = *P.step_base + 1;
    }
    if (a < P.nact) node_update<Q, S, MODE, KIND, WIDE, WALLS>(P, a, word, sp_entry, part);
    if constexpr (KIND == KIND_STEP) {
        if (!P.pdl_early) pdl_trigger();
    }
    if constexpr (KIND == KIND_READOUT) block_partials<BT>(part, P.partials);
}

// ---------------------------------------------------------------------------
// Compact step kernel: physics mode, FP32-arithmetic formats (FP32, FP16,
// BF16), 32-bit offsets, half-way bounce-back.  The same update as
// step_kernel (node_finish is shared, results are bit-identical), with the
// per-node 64-bit word and boundary-list entry (12 bytes a node) replaced
// by a block of words per warp of 32 consecutive active nodes: every lane
// derives its pull segment and its boundary-list entry from the warp's lane
// masks with a population count.  Pull offsets come from rows that already
// hold q * stride + delta_q, so a population's source index is one add (or,
// for a missing link, the node's own opposite population).
//
// Warp block (kWarpBlockWords words; warp w covers nodes 32 w .. 32 w + 31):
//   0 pull segment of lane 0's node
//   1 lane bit l (l >= 1): node l starts a new segment (segments are
//     numbered consecutively in active order)
//   2 next-to-wall lanes     3 wall and boundary-condition lanes
//   4 boundary-condition lanes
//   5 boundary-list entry of the first next-to-wall lane (next-to-wall
//     entries come first, in active order: lane l's entry is word 5 + the
//     next-to-wall lanes below l)
//   6 the same for the first wall / boundary-condition lane, counted from
//     the first entry after the next-to-wall ones
//   7 zero
// A lane's pull row (per-segment table) and a wall lane's missing-link mask
// (boundary list) wait on these words: lane masks -> row -> populations,
// the same three dependent loads as step_kernel's word -> row ->
// populations.  Measured on the 256x192x512 bifurcation: loading the warp's
// rows and masks beside the lane masks (prefetched to L1, or both rows in
// registers) did not shorten the step (FP32 30.7 / 37.1 us against 30.3 us,
// FP16 28.7 / 33.8 against 26.5 us), so the chain is not what bounds it.
template <int Q, typename S, int BT, int MINB>
__global__ void __launch_bounds__(BT, MINB) step_compact_kernel(const StepParams P) {
    using R = typename Store<S>::real;
    constexpr int DR = kDeltaRow<Q>, WB = kWarpBlockWords;
    double part[kPartialStride];
    uint32_t blk = blockIdx.x;
    if (P.pdl_early) pdl_trigger();
    if (blk < (uint32_t)P.fold_blocks) {
        // leading blocks: the stress ring's fold
        pdl_wait();
        if (blockIdx.x == 0 && threadIdx.x == 0) *P.step_next = *P.step_base + 1;
        fold_blocks_work(P, blk, BT);
        if (!P.pdl_early) pdl_trigger();
        return;
    }
    blk -= (uint32_t)P.fold_blocks;
    {
        // blocks from both ends of the active-node order first (step_kernel)
        const uint32_t nm = (uint32_t)((P.nact + BT - 1) / BT);
        blk = (blk & 1) ? nm - 1 - (blk >> 1) : (blk >> 1);
    }
    const uint32_t a = blk * BT + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31, bit = 1u << lane, below = bit - 1u;
    // read-only metadata before the dependency wait; the blocks cover whole
    // thread blocks (zero past the last node)
    const uint32_t* wb = P.warp_block + (size_t)WB * (a >> 5);
    const uint4 m0 = __ldg(reinterpret_cast<const uint4*>(wb));
    const uint4 m1 = __ldg(reinterpret_cast<const uint4*>(wb) + 1);
    const uint32_t kseg = __popc(m0.y & (below | bit));  // this lane's segment within the warp
    const bool nw = (m0.z & bit) != 0, ot = (m0.w & bit) != 0, bc = (m1.x & bit) != 0;
    int32_t s = 0;
    uint32_t miss = 0;
    float nr[3] = {0.f, 0.f, 0.f};
    if (nw) {
        s = (int32_t)(m1.y + __popc(m0.z & below));
        if (!in_bounds(s, P.nnw, P.flags)) s = 0;
        const int32_t ns = (int32_t)P.nw_stride;
        nr[0] = __ldg(P.nw_nf + s);
        nr[1] = __ldg(P.nw_nf + ns + s);
        nr[2] = __ldg(P.nw_nf + 2 * ns + s);
    }
    if (ot) {
        s = (int32_t)P.nnw + (int32_t)(m1.z + __popc(m0.w & below));
        if (!in_bounds(s, P.nsp, P.flags)) s = 0;
        miss = __ldg(P.sp_miss + s);
    }
    int32_t row[DR];
    {
        const uint32_t seg = in_bounds((int64_t)m0.x + kseg, P.nseg, P.flags) ? m0.x + kseg : 0u;
        const int4* r4 = reinterpret_cast<const int4*>(P.seg_abs + seg * DR);
#pragma unroll
        for (int k = 0; k < DR / 4; ++k) {
            const int4 v = __ldg(r4 + k);
            row[4 * k] = v.x; row[4 * k + 1] = v.y; row[4 * k + 2] = v.z; row[4 * k + 3] = v.w;
        }
    }
    pdl_wait();
    // block 0 is a node block when there are no fold blocks
    if (blockIdx.x == 0 && threadIdx.x == 0) *P.step_next = *P.step_base + 1;
    if (a < (uint32_t)P.nact) {
        const S* __restrict__ fin = static_cast<const S*>(P.fin);
        const uint32_t st = (uint32_t)P.stride;
        R g[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            uint32_t idx = a + (uint32_t)row[q];
            if (q != Lat<Q>::REST && (miss & (1u << Lat<Q>::opp(q)))) idx = a + (uint32_t)Lat<Q>::opp(q) * st;
            if (in_bounds(idx, (int64_t)Q * st, P.flags))
                g[q] = Store<S>::template load<Q>(fin + idx, q);  // w_opp(q) == w_q: the same decode
            else
                g[q] = R(0);
        }
        const int slot = nw ? (int)(*P.step_base & (kRingSlots - 1)) : 0;
        node_finish<Q, S, MODE_PHYSICS, KIND_STEP, false>(P, a, 0, s, nw || bc,
                                                           bc ? CLS_BC0 : (ot ? CLS_WALL : CLS_FLUID), miss, g, nr,
                                                           slot, part);
    }
    if (!P.pdl_early) pdl_trigger();
}

// Launch-shape variants of the step kernel, picked by the autotuner
// (lbm_autotune): block size and the minimum resident blocks per SM, which
// caps registers per thread at 65536 / (BT * MINB) -- more warps in flight
// on this latency-bound stencil against fewer registers (FP32 D3Q19 fits
// 40; D3Q27 and FP64 want more).
struct Variant {
    int bt, minb;
};
constexpr int kFlatVariants = 5;  // 0..4; 5 = tiled
constexpr Variant kVariants[kFlatVariants] = {{128, 12}, {128, 10}, {128, 8}, {256, 3}, {256, 1}};

// A step-kernel launch with programmatic stream serialization (see
// pdl_trigger / pdl_wait); minb: the kernel's minimum resident blocks per SM.
inline cudaError_t launch_dependent(void (*kern)(const StepParams), int64_t nblocks, int bt, int minb,
                                    const StepParams& p0, cudaStream_t st) {
    // SM count per device ordinal (handles on different devices may step
    // from different threads)
    constexpr int kDevs = 64;
    static std::atomic<int> sms_of[kDevs];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kDevs) return cudaErrorInvalidDevice;
    int sms = sms_of[dev].load(std::memory_order_acquire);
    if (sms <= 0) {
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        sms_of[dev].store(sms, std::memory_order_release);
    }
    StepParams p = p0;
    p.pdl_early = nblocks > (int64_t)minb * sms ? 1 : 0;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)nblocks);
    cfg.blockDim = dim3(bt);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, p);
}

template <int Q, typename S, int MODE, int V>
cudaError_t launch_step_variant(const StepParams& p, cudaStream_t st) {
    constexpr int BT = kVariants[V].bt, MB = kVariants[V].minb;
    const bool narrow = (int64_t)Q * p.stride < ((int64_t)1 << 31);
    const int bt = narrow ? BT : kStepThreads;  // beyond 32-bit offsets: one 64-bit shape for every variant
    constexpr bool PHYS = MODE == MODE_PHYSICS;
    const bool walls = PHYS && p.sp_q != nullptr;  // interpolated bounce-back: one shape, (128, 8)
    const int bw = walls && narrow ? 128 : bt;
    StepParams q = p;
    q.fold_blocks = Store<S>::offset ? ceil_div(p.nnw, (int64_t)bw * kFoldNodes) : 0;
    const int64_t nblocks = q.fold_blocks + ceil_div(p.nact, bw);
    if (ceil_div(p.nact, bw) <= 0) return cudaSuccess;
    if (nblocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    if (walls) {
        if constexpr (PHYS) {
            if (narrow)
                return launch_dependent(step_kernel<Q, S, MODE, KIND_STEP, 128, 8, false, true>, nblocks, 128, 8, q,
                                        st);
            return launch_dependent(step_kernel<Q, S, MODE, KIND_STEP, kStepThreads, 1, true, true>, nblocks,
                                    kStepThreads, 1, q, st);
        }
        return cudaErrorInvalidValue;
    }
    if (narrow) return launch_dependent(step_kernel<Q, S, MODE, KIND_STEP, BT, MB, false>, nblocks, BT, MB, q, st);
    return launch_dependent(step_kernel<Q, S, MODE, KIND_STEP, kStepThreads, 1, true>, nblocks, kStepThreads, 1, q,
                            st);
}

// ---------------------------------------------------------------------------
// Persistent multi-step kernel (small lattices and ensembles of small
// vessels, where a step is shorter than a launch): one cooperative launch of
// at most as many blocks as are resident at once runs nsteps steps, each
// thread walking the nodes with a grid stride, with a grid barrier between
// steps.  PP.p[0] / PP.p[1] are the parameters of the launch's even / odd
// steps (buffer roles and counter slots swap each step).  Populations and
// the stress ring are read from L2 (Store::load CG): they were written by
// other SMs earlier in the same launch.  Every barrier wait is bounded: a
// block that gives up raises FLAG_TIMEOUT and returns, after which every
// other block gives up at its next barrier too.
//
// Barrier word bar[0] counts arrivals over the whole launch: barrier j of a
// grid of n blocks completes when it reaches (j + 1) n (+ bar[1], zero
// except when a test asks for a barrier that cannot complete).  Arrival is
// a release add, the wait an acquire poll: the release orders this block's
// writes (made visible to its thread 0 by the preceding __syncthreads)
// before the arrival, the acquire orders the other blocks' writes before
// this block's next loads.  Each block adds 1 more when it leaves; the last
// to leave stores 0, so the next launch starts from zero.  The host clears
// both words when it reads FLAG_TIMEOUT.

constexpr long kBarrierPolls = 1L << 20;  // L2 reads: well under a second

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Returns false when the wait gave up.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned target, unsigned* flags) {
    __shared__ int passed;
    __syncthreads();
    if (threadIdx.x == 0) {
        red_release_add(bar, 1u);
        const unsigned goal = target + ld_acquire(bar + 1);
        int ok = 0;
        for (long it = 0; it < kBarrierPolls; ++it) {
            if ((int)(ld_acquire(bar) - goal) >= 0) {
                ok = 1;
                break;
            }
        }
        if (!ok) atomicOr(flags, FLAG_TIMEOUT);
        passed = ok;
    }
    __syncthreads();
    return passed != 0;
}

// The launch's last block to leave resets the arrival count.
__device__ __forceinline__ void grid_leave(unsigned* bar, unsigned total) {
    if (threadIdx.x == 0 && atomicAdd(bar, 1u) == total - 1) atomicExch(bar, 0u);
}

struct StepPair {
    StepParams p[2];
};

constexpr int kMultiThreads = 256;

// minimum resident blocks per SM: register caps of 255 (FP64), 128 (D3Q27)
// and 64 (D3Q19 FP32 / FP16 / BF16) registers a thread, the largest blocks
// per SM that do not spill (the grid-stride loop keeps more live state than
// the flat kernel's 40 registers)
template <int Q, typename S>
constexpr int multi_min_blocks() {
    return std::is_same<S, double>::value ? 1 : (Q == 27 ? 2 : 4);
}

template <int Q, typename S, int MODE, bool WALLS>
__global__ void __launch_bounds__(kMultiThreads, multi_min_blocks<Q, S>())
    step_kernel_multi(const StepPair PP, int nsteps, unsigned* bar) {
    double part[kPartialStride];
    const int64_t T = (int64_t)gridDim.x * kMultiThreads;
    const int64_t t0 = (int64_t)blockIdx.x * kMultiThreads + threadIdx.x;
    for (int k = 0; k < nsteps; ++k) {
        const StepParams& P = PP.p[k & 1];
        const int64_t step = __ldcg(P.step_base);
        if (t0 == 0) *P.step_next = step + 1;
        if constexpr (Store<S>::offset) {
            // the stress ring's fold, as the fold blocks of a flat launch do it
            if (step % kFoldEvery == 0) {
                const int writing = (int)((step % kRingSlots) / kFoldEvery);
                for (int64_t nw = t0; nw < P.nnw; nw += T) fold_half<true>(P, nw, 1 - writing);
            }
        }
        for (int64_t a = t0; a < P.nact; a += T)
            node_update<Q, S, MODE, KIND_STEP, false, WALLS, true>(P, a, __ldg(P.act_word + a),
                                                                  __ldg(P.sp_of_act + a), part);
        if (k + 1 < nsteps && !grid_barrier(bar, (unsigned)(k + 1) * gridDim.x, P.flags)) return;
    }
    grid_leave(bar, (unsigned)nsteps * gridDim.x);
}

template <int Q, typename S, int MODE, bool WALLS>
cudaError_t launch_multi_t(const StepPair& pp, int nsteps, unsigned* bar, cudaStream_t st) {
    auto kern = step_kernel_multi<Q, S, MODE, WALLS>;
    // resident blocks per SM of this instantiation and SM count, per device
    // ordinal (handles on different devices may step from different threads)
    constexpr int kDevs = 64;
    static std::atomic<int> per_sm_of[kDevs];
    static std::atomic<int> sms_of[kDevs];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kDevs) return cudaErrorInvalidDevice;
    int per_sm = per_sm_of[dev].load(std::memory_order_acquire);
    int sms = sms_of[dev].load(std::memory_order_acquire);
    if (per_sm <= 0 || sms <= 0) {
        int v = 0, n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, kMultiThreads, 0);
        if (e != cudaSuccess) return e;
        if (v <= 0 || n <= 0) return cudaErrorInvalidConfiguration;
        sms = n;
        per_sm = v;
        sms_of[dev].store(n, std::memory_order_release);
        per_sm_of[dev].store(v, std::memory_order_release);
    }
    if (nsteps == 0) return cudaSuccess;  // the occupancy query alone (before a stream capture)
    const StepParams& p = pp.p[0];
    const int64_t work = p.nact > p.nnw ? p.nact : p.nnw;
    const int64_t need = ceil_div(work, kMultiThreads);
    const int64_t full = (int64_t)per_sm * sms;
    const unsigned nb = (unsigned)(need < 1 ? 1 : (need < full ? need : full));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(kMultiThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, pp, nsteps, bar);
}

// nsteps steps in one launch (0: only the kernel's occupancy query, which
// is then done outside any stream capture); lattices with 32-bit
// population offsets only.
template <typename S>
cudaError_t launch_multi_typed(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                               unsigned* bar, cudaStream_t st) {
    if ((int64_t)Q * even.stride >= ((int64_t)1 << 31) || nsteps < 0) return cudaErrorInvalidValue;
    if (even.nact <= 0) return cudaSuccess;
    StepPair pp{};
    pp.p[0] = even;
    pp.p[1] = odd;
    pp.p[0].fold_blocks = pp.p[1].fold_blocks = 0;
    const bool walls = mode == MODE_PHYSICS && even.sp_q != nullptr;
    if (Q == 19) {
        if (mode == MODE_PARITY) return launch_multi_t<19, S, MODE_PARITY, false>(pp, nsteps, bar, st);
        return walls ? launch_multi_t<19, S, MODE_PHYSICS, true>(pp, nsteps, bar, st)
                     : launch_multi_t<19, S, MODE_PHYSICS, false>(pp, nsteps, bar, st);
    }
    if (mode == MODE_PARITY) return launch_multi_t<27, S, MODE_PARITY, false>(pp, nsteps, bar, st);
    return walls ? launch_multi_t<27, S, MODE_PHYSICS, true>(pp, nsteps, bar, st)
                 : launch_multi_t<27, S, MODE_PHYSICS, false>(pp, nsteps, bar, st);
}

// ---------------------------------------------------------------------------
// Tiled step.  A tile is kTileNodes consecutive active nodes; in active-index
// order the pull sources of a tile's nodes for population q lie in one
// contiguous window of plane q (measured on the bifurcation: about the tile's
// own size), so one bulk copy per plane (cp.async.bulk, the TMA engine)
// stages all of them in shared memory, with the tile's own entries of every
// plane (bounce-back reads them), its node words, boundary-list entries,
// delta rows and next-to-wall normals.  Persistent CTAs of kTileNodes
// threads loop over tiles; an mbarrier per stage tracks the copies, NS
// stages deep, so a tile's loads fly while earlier tiles compute.  Every
// wait is bounded: a copy that does not land raises FLAG_TIMEOUT, the CTA
// waits (bounded) for what it issued and returns.

constexpr int64_t kWaitLimit = 1 << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// false when the phase did not complete within the limit
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int64_t k = 0; k < kWaitLimit; ++k)
        if (mbar_test(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Issue every copy of tile t into one stage (one thread).  Sizes and
// alignments come from the plan: windows start and end on 16-byte
// boundaries inside their planes.
template <int Q, typename S>
__device__ __forceinline__ void tile_issue(const StepParams& P, int64_t t, unsigned char* sb, uint64_t* bar) {
    constexpr int T = kTileNodes, DR = kDeltaRow<Q>;
    const TileGeom& G = P.tile;
    const int32_t* pl = P.tile_plan + t * (2 * Q + kTilePlanExtra);
    const S* fin = static_cast<const S*>(P.fin);
    int32_t* hdr = reinterpret_cast<int32_t*>(sb + G.off_hdr);
    const int64_t t0 = t * T;
    const int nt = (int)(P.nact - t0 < T ? P.nact - t0 : T);
    const int nown = (int)(P.stride - t0 < T ? P.stride - t0 : T);
    const int seg0 = pl[2 * Q], nseg = pl[2 * Q + 1], nw0 = pl[2 * Q + 2], nwl = pl[2 * Q + 3];
    const int nword = (nt + 1) & ~1, nsp = (nt + 3) & ~3;
    uint32_t bytes = (uint32_t)(Q * nown * (int)sizeof(S) + nword * 8 + nsp * 4 + nseg * DR * 4 + 3 * nwl * 4);
    for (int q = 0; q < Q; ++q) {
        hdr[q] = pl[q];
        bytes += (uint32_t)(pl[Q + q] * (int)sizeof(S));
    }
    hdr[Q] = seg0;
    hdr[Q + 1] = nseg;
    hdr[Q + 2] = nw0;
    // the previous tile's reads of this stage (generic proxy) before the
    // copies (async proxy) overwrite it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_tx(bar, bytes);
    S* pull = reinterpret_cast<S*>(sb + G.off_pull);
    S* own = reinterpret_cast<S*>(sb + G.off_own);
    for (int q = 0; q < Q; ++q) {
        if (pl[Q + q] > 0)
            bulk_load(pull + (int64_t)q * G.wcap, fin + (int64_t)q * P.stride + pl[q], (uint32_t)(pl[Q + q] * sizeof(S)),
                      bar);
        bulk_load(own + q * T, fin + (int64_t)q * P.stride + t0, (uint32_t)(nown * sizeof(S)), bar);
    }
    bulk_load(sb + G.off_word, P.act_word + t0, (uint32_t)(nword * 8), bar);
    bulk_load(sb + G.off_sp, P.sp_of_act + t0, (uint32_t)(nsp * 4), bar);
    if (nseg > 0) bulk_load(sb + G.off_delta, P.seg_delta + (int64_t)seg0 * DR, (uint32_t)(nseg * DR * 4), bar);
    if (nwl > 0)
        for (int k = 0; k < 3; ++k)
            bulk_load(sb + G.off_nrm + k * G.nwcap * 4, P.nw_nf + k * P.nw_stride + nw0, (uint32_t)(nwl * 4), bar);
}

// Physics mode, FP32-arithmetic formats, 32-bit offsets.
template <int Q, typename S, int NS>
__global__ void __launch_bounds__(kTileNodes, 1) tile_step_kernel(const StepParams P) {
    using R = typename Store<S>::real;
    constexpr int T = kTileNodes, DR = kDeltaRow<Q>;
    const TileGeom& G = P.tile;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + NS * G.stage_bytes);
    const int tid = threadIdx.x;
    const int64_t grid = gridDim.x;
    int issued[NS], used[NS];  // phases issued / consumed per stage (thread 0 issues)
#pragma unroll
    for (int k = 0; k < NS; ++k) issued[k] = used[k] = 0;
    if (tid == 0) {
        for (int k = 0; k < NS; ++k) mbar_init(&bar[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < NS - 1; ++k) {
            const int64_t t = blockIdx.x + k * grid;
            if (t < G.ntiles) {
                tile_issue<Q, S>(P, t, smem + k * G.stage_bytes, &bar[k]);
                ++issued[k];
            }
        }
    double part[kPartialStride];
    bool failed = false;
    int it = 0;
    for (int64_t t = blockIdx.x; t < G.ntiles; t += grid, ++it) {
        const int stg = it % NS;
        if (tid == 0) {
            const int64_t tn = t + (int64_t)(NS - 1) * grid;
            const int sn = (it + NS - 1) % NS;
            if (tn < G.ntiles) {
                tile_issue<Q, S>(P, tn, smem + sn * G.stage_bytes, &bar[sn]);
                ++issued[sn];
            }
        }
        const bool ok = mbar_wait(&bar[stg], (uint32_t)(used[stg] & 1));
        ++used[stg];
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        const unsigned char* sb = smem + stg * G.stage_bytes;
        const int32_t* hdr = reinterpret_cast<const int32_t*>(sb + G.off_hdr);
        const int64_t a = t * T + tid;
        if (a < P.nact) {
            const uint64_t word = reinterpret_cast<const uint64_t*>(sb + G.off_word)[tid];
            const int32_t sp_entry = reinterpret_cast<const int32_t*>(sb + G.off_sp)[tid];
            const uint32_t miss = word_miss(word);
            const int c = word_class(word);
            const bool lng = c >= CLS_BC0 || word_nw(word);
            const int64_t s = lng ? (int64_t)sp_entry : 0;
            float nr[3] = {0.f, 0.f, 0.f};
            int slot = 0;
            if (lng && s < P.nnw) {
                const float* nrm = reinterpret_cast<const float*>(sb + G.off_nrm);
                const int k = (int)(s - hdr[Q + 2]);
                nr[0] = nrm[k];
                nr[1] = nrm[G.nwcap + k];
                nr[2] = nrm[2 * G.nwcap + k];
                slot = (int)(*P.step_base % kRingSlots);
            }
            int32_t dl[DR];
            const int64_t rs = word_segment(word) - hdr[Q];
            const int4* drow = (rs >= 0 && rs < hdr[Q + 1])
                                   ? reinterpret_cast<const int4*>(sb + G.off_delta) + rs * (DR / 4)
                                   : reinterpret_cast<const int4*>(P.seg_delta + word_segment(word) * DR);
#pragma unroll
            for (int k = 0; k < DR / 4; ++k) {
                const int4 v = drow[k];
                dl[4 * k] = v.x; dl[4 * k + 1] = v.y; dl[4 * k + 2] = v.z; dl[4 * k + 3] = v.w;
            }
            const S* pull = reinterpret_cast<const S*>(sb + G.off_pull);
            const S* own = reinterpret_cast<const S*>(sb + G.off_own);
            R g[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                S v;
                if (q == Lat<Q>::REST) v = own[q * T + tid];
                else if ((miss >> Lat<Q>::opp(q)) & 1u) v = own[Lat<Q>::opp(q) * T + tid];
                else v = pull[q * G.wcap + (int)(a + dl[q] - hdr[q])];
                g[q] = Store<S>::template decode<Q>(v, q);
            }
            node_finish<Q, S, MODE_PHYSICS, KIND_STEP, false>(P, a, word, s, lng, c, miss, g, nr, slot, part);
        }
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) {
            atomicOr(P.flags, FLAG_TIMEOUT);
            // wait, bounded, for the copies this CTA still has in flight
            for (int k = 0; k < NS; ++k)
                for (; used[k] < issued[k]; ++used[k])
                    if (!mbar_wait(&bar[k], (uint32_t)(used[k] & 1))) break;
        }
        __syncthreads();
        return;
    }
    if (blockIdx.x == 0 && tid == 0) *P.step_next = *P.step_base + 1;
}

template <int Q, typename S, int NS>
cudaError_t launch_tile_ns(const StepParams& p, cudaStream_t st) {
    // per instantiation and device ordinal: opt-in shared memory set so far
    constexpr int kDevs = 64;
    static std::atomic<int> attr_bytes[kDevs];
    int dev = 0, nsm = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kDevs) return cudaErrorInvalidDevice;
    if (p.tile.smem_bytes > attr_bytes[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(tile_step_kernel<Q, S, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p.tile.smem_bytes);
        if (e != cudaSuccess) return e;
        attr_bytes[dev].store(p.tile.smem_bytes, std::memory_order_release);
    }
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
    int64_t grid = (int64_t)nsm * p.tile.ctas_per_sm;
    if (grid > p.tile.ntiles) grid = p.tile.ntiles;
    tile_step_kernel<Q, S, NS><<<(unsigned)grid, kTileNodes, p.tile.smem_bytes, st>>>(p);
    return cudaGetLastError();
}

template <int Q, typename S>
cudaError_t launch_tile(const StepParams& p, cudaStream_t st) {
    cudaError_t e = p.tile.nstage == 3 ? launch_tile_ns<Q, S, 3>(p, st) : launch_tile_ns<Q, S, 2>(p, st);
    // the tiled kernel has no fold blocks: the stress ring's fold follows it
    if (e == cudaSuccess && p.nnw > 0) {
        k_fold_ring<<<(unsigned)ceil_div(p.nnw, 256), 256, 0, st>>>(p);
        e = cudaGetLastError();
    }
    return e;
}

// The compact kernel where its warp blocks exist (physics, FP32-arithmetic
// formats, 32-bit offsets, half-way bounce-back); the flat kernel's default
// shape elsewhere.
template <int Q, typename S, int MODE, int BT, int MB>
cudaError_t launch_compact(const StepParams& p, cudaStream_t st) {
    if constexpr (Store<S>::offset && MODE == MODE_PHYSICS) {
        if (p.warp_block && p.seg_abs && !p.sp_q && (int64_t)Q * p.stride < ((int64_t)1 << 31)) {
            StepParams q = p;
            q.fold_blocks = ceil_div(p.nnw, (int64_t)BT * kFoldNodes);
            const int64_t nb = ceil_div(p.nact, BT);
            if (nb <= 0) return cudaSuccess;
            return launch_dependent(step_compact_kernel<Q, S, BT, MB>, q.fold_blocks + nb, BT, MB, q, st);
        }
    }
    return launch_step_variant<Q, S, MODE, 0>(p, st);
}

template <int Q, typename S, int MODE>
cudaError_t launch_family(int kind, int variant, const StepParams& p, cudaStream_t st) {
    if (kind == KIND_STEP) {
        switch (variant) {
            case 1: return launch_step_variant<Q, S, MODE, 1>(p, st);
            case 2: return launch_step_variant<Q, S, MODE, 2>(p, st);
            case 3: return launch_step_variant<Q, S, MODE, 3>(p, st);
            case 4: return launch_step_variant<Q, S, MODE, 4>(p, st);
            case 6: return launch_compact<Q, S, MODE, 128, 10>(p, st);
            case 7: return launch_compact<Q, S, MODE, 128, 12>(p, st);
            case 5:
                // the tiled kernel where a plan exists (physics, FP32-arithmetic
                // formats, 32-bit offsets, half-way bounce-back); the default
                // shape elsewhere
                if constexpr (Store<S>::offset && MODE == MODE_PHYSICS) {
                    if (p.tile.ntiles > 0 && p.tile_plan && !p.sp_q && (int64_t)Q * p.stride < ((int64_t)1 << 31))
                        return launch_tile<Q, S>(p, st);
                }
                return launch_step_variant<Q, S, MODE, Store<S>::offset ? 0 : 4>(p, st);
            default: return launch_step_variant<Q, S, MODE, 0>(p, st);
        }
    }
    // prologue and read-out: default shape (the read-out's partial sums are per 256-thread block)
    const int64_t nblocks = ceil_div(p.nact, kStepThreads);
    if (nblocks <= 0) return cudaSuccess;
    if (nblocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    if (kind == KIND_PROLOGUE) {
        step_kernel<Q, S, MODE, KIND_PROLOGUE><<<(unsigned)nblocks, kStepThreads, 0, st>>>(p);
    } else if (MODE == MODE_PHYSICS && p.sp_q != nullptr) {
        // the read-out's pull applies the same interpolated bounce-back
        if constexpr (MODE == MODE_PHYSICS)
            step_kernel<Q, S, MODE, KIND_READOUT, kStepThreads, 1, true, true>
                <<<(unsigned)nblocks, kStepThreads, 0, st>>>(p);
    } else {
        step_kernel<Q, S, MODE, KIND_READOUT><<<(unsigned)nblocks, kStepThreads, 0, st>>>(p);
    }
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_typed(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t st) {
    if (Q == 19) {
        return mode == MODE_PARITY ? launch_family<19, S, MODE_PARITY>(kind, variant, p, st)
                                   : launch_family<19, S, MODE_PHYSICS>(kind, variant, p, st);
    }
    return mode == MODE_PARITY ? launch_family<27, S, MODE_PARITY>(kind, variant, p, st)
                               : launch_family<27, S, MODE_PHYSICS>(kind, variant, p, st);
}

// ---------------------------------------------------------------------------
// State initialisation kernels (storage-typed).

template <int Q, typename S>
__device__ __forceinline__ S encode_full(double f, int q) {
    using R = typename Store<S>::real;
    if constexpr (Store<S>::scaled)
        return Store<S>::template pack<Q>((R)((f - Lat<Q>::w(q)) / (double)Store<S>::template unit<Q>(q)), q);
    else if constexpr (Store<S>::offset)
        return Store<S>::template pack<Q>((R)(f - Lat<Q>::w(q)), q);
    else
        return Store<S>::template pack<Q>((R)f, q);
}

// Every plane entry of every active node := f = w (Node.cpp:30-37).
template <int Q, typename S>
__global__ void k_fill_weights(S* __restrict__ f, int64_t stride, int64_t nact) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nact) return;
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q * stride + a] = encode_full<Q, S>(Lat<Q>::w(q), q);
}

// fa[a*Q + q] (FP64 f, per active node) into the planes.
template <int Q, typename S>
__global__ void k_scatter_f(const double* __restrict__ fa, int64_t nact, S* __restrict__ f, int64_t stride) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nact) return;
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q * stride + a] = encode_full<Q, S>(fa[a * Q + q], q);
}

template <typename S>
cudaError_t init_typed(int Q, int what, void* f, int64_t stride, const double* fa, int64_t nact, cudaStream_t st) {
    const unsigned g = (unsigned)ceil_div(nact > 0 ? nact : 1, 256);
    if (what == 0) {
        if (Q == 19) k_fill_weights<19, S><<<g, 256, 0, st>>>(static_cast<S*>(f), stride, nact);
        else k_fill_weights<27, S><<<g, 256, 0, st>>>(static_cast<S*>(f), stride, nact);
    } else {
        if (Q == 19) k_scatter_f<19, S><<<g, 256, 0, st>>>(fa, nact, static_cast<S*>(f), stride);
        else k_scatter_f<27, S><<<g, 256, 0, st>>>(fa, nact, static_cast<S*>(f), stride);
    }
    return cudaGetLastError();
}

}  // namespace lbm
