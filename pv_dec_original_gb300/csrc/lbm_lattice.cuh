// Lattice tables and storage traits shared by every kernel.
//
// Direction numbering follows the reference so that distributions, boundary
// formulas and dumps line up index for index:
//   D3Q19: LatticeModel.cpp:51-151 (rest population is index 18),
//   D3Q27: LatticeModel.cpp:208-334 (rest population is index 0).
// Weights are the reference's literals (2/36, 1/36, 12/36; 8/27, 2/27, 1/54,
// 1/216) so host and device produce identical doubles.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

namespace lbm {

template <int Q> struct Lat;

template <> struct Lat<19> {
    static constexpr int Q = 19;
    static constexpr int REST = 18;
    __host__ __device__ static constexpr int cx(int q) {
        constexpr int t[19] = {1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0, 0};
        return t[q];
    }
    __host__ __device__ static constexpr int cy(int q) {
        constexpr int t[19] = {0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0};
        return t[q];
    }
    __host__ __device__ static constexpr int cz(int q) {
        constexpr int t[19] = {0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 0};
        return t[q];
    }
    __host__ __device__ static constexpr int opp(int q) {
        constexpr int t[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};
        return t[q];
    }
    __host__ __device__ static constexpr double w(int q) {
        return q < 6 ? 2.0 / 36.0 : (q < 18 ? 1.0 / 36.0 : 12.0 / 36.0);
    }
    // Sum over the unknown populations of one face of c_t^2 for a transverse axis t.
    static constexpr double ZH_M = 2.0;
};

template <> struct Lat<27> {
    static constexpr int Q = 27;
    static constexpr int REST = 0;
    __host__ __device__ static constexpr int cx(int q) {
        constexpr int t[27] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
        return t[q];
    }
    __host__ __device__ static constexpr int cy(int q) {
        constexpr int t[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 1, -1, -1, 1, -1, 1};
        return t[q];
    }
    __host__ __device__ static constexpr int cz(int q) {
        constexpr int t[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1, -1, 1};
        return t[q];
    }
    __host__ __device__ static constexpr int opp(int q) {
        constexpr int t[27] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15,
                               20, 19, 22, 21, 24, 23, 26, 25};
        return t[q];
    }
    __host__ __device__ static constexpr double w(int q) {
        return q == 0 ? 8.0 / 27.0 : (q < 7 ? 2.0 / 27.0 : (q < 19 ? 1.0 / 54.0 : 1.0 / 216.0));
    }
    static constexpr double ZH_M = 6.0;
};

template <int Q>
__host__ __device__ constexpr int lat_c(int q, int axis) {
    return axis == 0 ? Lat<Q>::cx(q) : (axis == 1 ? Lat<Q>::cy(q) : Lat<Q>::cz(q));
}

// ---------------------------------------------------------------------------
// Storage formats and the arithmetic value they hold.
//
// FP64: f itself, FP64 arithmetic in the reference's operation order.
// FP32, FP16, BF16: the offset d = f - w from the lattice weight, with all
// arithmetic in FP32 on d (the collision, Zou-He and stress formulas are
// affine in f and are written for d).  Near rest |d| << w, so carrying d
// keeps ~5 more significant bits than carrying f.  Storage of d:
//   FP32: d,            FP16: d / w * 1024,          BF16: d / w.
// The relative scaling by 1/w gives every direction the same range; the
// factor 1024 keeps FP16 offsets down to ~6e-8 normal while +-0.5 relative
// offsets stay far below the FP16 maximum.  BF16 has FP32's exponent range.
// FP16 and BF16 ("scaled") keep their storage units g = d / unit_q through
// the collision (unit_q = w_q / 1024 and w_q): a load or store is a bare
// conversion, the moments weight g by unit_q (a multiply-add in place of an
// add), and the equilibrium in these units, (w_q / unit_q) (B + ...), has
// the same factor geq (1024, 1) for every direction.
// load<Q, CG>: CG = false reads through the non-coherent (read-only) path,
// valid while no thread of the launch writes the buffer; CG = true reads
// from L2 (ld.global.cg), for a persistent launch whose steps read what its
// earlier steps wrote.
enum Precision : int { P_F64 = 0, P_F32 = 1, P_F16 = 2, P_BF16 = 3 };

template <typename S> struct Store;

template <> struct Store<double> {
    using real = double;
    static constexpr bool offset = false;
    static constexpr bool scaled = false;
    template <int Q, bool CG = false>
    __device__ static __forceinline__ real load(const double* p, int q) { return CG ? __ldcg(p) : *p; }
    template <int Q>
    __device__ static __forceinline__ real decode(double v, int q) { return v; }
    template <int Q>
    __device__ static __forceinline__ double pack(real f, int q) { return f; }
};

template <> struct Store<float> {
    using real = float;
    static constexpr bool offset = true;
    static constexpr bool scaled = false;
    template <int Q, bool CG = false>
    __device__ static __forceinline__ real load(const float* p, int q) { return CG ? __ldcg(p) : __ldg(p); }
    template <int Q>
    __device__ static __forceinline__ real decode(float v, int q) { return v; }
    template <int Q>
    __device__ static __forceinline__ float pack(real d, int q) { return d; }
};

template <> struct Store<__half> {
    using real = float;
    static constexpr bool offset = true;
    static constexpr bool scaled = true;
    static constexpr float S = 1024.0f;
    static constexpr float geq = S;  // w_q / unit_q
    template <int Q>
    __host__ __device__ static constexpr float unit(int q) { return (float)(Lat<Q>::w(q) / 1024.0); }
    template <int Q, bool CG = false>
    __device__ static __forceinline__ real load(const __half* p, int q) {
        return __half2float(CG ? __ldcg(p) : __ldg(p));
    }
    template <int Q>
    __device__ static __forceinline__ real decode(__half v, int q) { return __half2float(v); }
    template <int Q>
    __device__ static __forceinline__ __half pack(real g, int q) { return __float2half_rn(g); }
};

template <> struct Store<__nv_bfloat16> {
    using real = float;
    static constexpr bool offset = true;
    static constexpr bool scaled = true;
    static constexpr float geq = 1.0f;
    template <int Q>
    __host__ __device__ static constexpr float unit(int q) { return (float)Lat<Q>::w(q); }
    template <int Q, bool CG = false>
    __device__ static __forceinline__ real load(const __nv_bfloat16* p, int q) {
        return __bfloat162float(CG ? __ldcg(p) : __ldg(p));
    }
    template <int Q>
    __device__ static __forceinline__ real decode(__nv_bfloat16 v, int q) { return __bfloat162float(v); }
    template <int Q>
    __device__ static __forceinline__ __nv_bfloat16 pack(real g, int q) { return __float2bfloat16_rn(g); }
};

}  // namespace lbm
