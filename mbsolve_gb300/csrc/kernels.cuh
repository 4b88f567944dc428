// Time-step kernels of the Maxwell-Bloch loop.
//
// One kernel launch advances every tile of every run by up to `nsub` time
// steps (temporal blocking). A CTA owns NT*C consecutive grid points of one
// run, C per thread in registers, and keeps them on chip for all sub-steps:
//   state in  : [out_start - halo, out_start + out_len + halo)
//   state out : [out_start, out_start + out_len)
// Each sub-step reproduces one iteration of solver_cpu_fdtd::run
// (solver-cpu/include/mbsolve/solver-cpu/solver_cpu_fdtd.tpp:223-325):
//   E[i] = a E[i] + b (-Gamma P[i] + (H[i+1] - H[i]) / dx)      (:238-243)
//   hard/soft sources on E                                       (:247-255)
//   H[i] += c (E[i] - E[i-1]), i >= 1; H[0] = H[N] = 0          (:263-275)
//   density update and P[i] = dP/dt at every point              (:279-285)
//   recording                                                    (:288-325)
// Neighbour values cross thread boundaries by warp shuffles and cross warp
// boundaries through shared memory (two barriers per step). Garbage from
// the tile edges moves one point per step, so after `nsub <= halo` steps
// the output range is exact. Points outside the run keep zero state (the
// one-point loop never updates them; the packed-pair loop of uniform
// 2-level FP32 tiles, pair_steps.cuh, updates them with their neighbours
// and puts them back after each step); the reference's index rules (no H
// update at i = 0, H[N] = 0) give them no influence on the run.
//
// FP32 kernels keep the density state, and E and H in all but the 2-level
// kernel, as unevaluated sums hi + lo of two floats updated with
// error-free transformations (TwoSum; TwoProd by fma): the spatial
// differences of FP32 fields lose about log2(points per wavelength) bits,
// and the per-step rounding of small density increments accumulates; with
// the float pairs the FP32 result tracks the FP64 one to ~1e-7 while
// polarisation and all matrix work stay in FP32. The 2-level kernel keeps
// E and H in plain FP32 (one rounding per update by fma): ~6e-6 over 1e5
// steps, within the 1e-5 target, for 22 % more throughput; on uniform
// tiles it updates two points per instruction (packed FP32 pairs, the
// same roundings).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "common.cuh"
#include "precompute.cuh"

namespace mbg {

template<typename T>
struct kparams {
    const T* Ein;
    const T* Hin;
    const T* Pin;
    const T* Din;  // density planes, `plane` apart
    const T* Elin; // FP32 only: low parts of E and H (double-float fields)
    const T* Hlin;
    T* Eout;
    T* Hout;
    T* Pout;
    T* Dout;
    T* Elout;
    T* Hlout;
    uint64_t plane;
    const int32_t* mat;  // global material index per point (-1: none)
    const T* mc;         // material constant blocks
    uint32_t mstride;
    uint32_t mstage;     // leading entries of a block staged in shared memory
    const tile_desc* tiles;
    const run_desc* runs;
    const src_desc* srcs;
    const double* stab;  // source value tables (FP64)
    const rec_desc* recs;
    T* scratch;
    const unsigned long long* step_base;  // device step counter
    uint32_t launch_idx;  // step0 = *step_base + launch_idx * depth
    uint32_t depth;
    uint32_t nsub;        // sub-steps of this launch (<= depth)
    uint32_t halo;
    int record;           // 0 while autotuning
    uint32_t* status;
    uint32_t wait_limit;  // polls of a bounded device wait (0: the kernel's default)
};

// ------------------------------------------------------------ helpers

// sin(x) and 1 - cos(x). For small |x| by their Taylor series (enough
// terms for the type's precision: truncation below 1e-10 relative in
// float, 1e-30 in double); beyond that by the library sincos.
template<typename T>
__device__ __forceinline__ void rot_coeffs(T x, T& s, T& s2);

template<>
__device__ __forceinline__ void rot_coeffs<float>(float x, float& s, float& s2)
{
    // |x| < 1/128 (the field rotation per step in the workloads here is
    // ~1e-3): sin x = x - x^3/6, 1 - cos x = x^2/2 - x^4/24; the first
    // omitted terms (x^4/120 and x^4/360 of the result) are below 4e-11 of
    // it, over 1000 times below half an FP32 ulp
    if (fabsf(x) < 0.0078125f) {
        const float x2 = x * x;
        s = fmaf(x * x2, -1.0f / 6.0f, x);
        s2 = x2 * fmaf(x2, -1.0f / 24.0f, 0.5f);
    } else if (fabsf(x) < 0.0625f) {
        // |x| < 1/16: the series to x^7 and x^8, Horner in x^2; the first
        // omitted terms are below 1e-14 of the result
        const float x2 = x * x;
        // sin x = x (1 - x^2/3! + x^4/5! - x^6/7!)
        float t = fmaf(x2, -1.0f / 5040.0f, 1.0f / 120.0f);
        t = fmaf(x2, t, -1.0f / 6.0f);
        s = fmaf(x * x2, t, x);
        // 1 - cos x = x^2/2! - x^4/4! + x^6/6! - x^8/8!
        float u = fmaf(x2, 1.0f / 40320.0f, -1.0f / 720.0f);
        u = fmaf(x2, u, 1.0f / 24.0f);
        u = fmaf(x2, -u, 0.5f);
        s2 = x2 * u;
    } else {
        float c;
        sincosf(x, &s, &c);
        s2 = 1.0f - c;
    }
}

template<>
__device__ __forceinline__ void rot_coeffs<double>(double x, double& s, double& s2)
{
    if (fabs(x) < 0.25) {
        double x2 = x * x;
        double t = 1.0, u = 1.0;
#pragma unroll
        for (int k = 10; k >= 1; k--) {
            t = 1.0 - x2 / ((2.0 * k) * (2.0 * k + 1.0)) * t;
            u = 1.0 - x2 / ((2.0 * k + 1.0) * (2.0 * k + 2.0)) * u;
        }
        s = x * t;
        s2 = 0.5 * x2 * u;
    } else {
        double c;
        sincos(x, &s, &c);
        s2 = 1.0 - c;
    }
}

// CG: through L2 only (data another CTA of the same launch wrote);
// otherwise streaming loads
template<typename T, int C, bool CG = false>
__device__ __forceinline__ void load_cells(T (&r)[C], const T* __restrict__ src, int64_t g0)
{
    if constexpr (sizeof(T) == 4 && (C % 4) == 0) {
        const float4* s4 = reinterpret_cast<const float4*>(src + g0);
#pragma unroll
        for (int q = 0; q < C / 4; q++) {
            float4 v = CG ? __ldcg(s4 + q) : __ldcs(s4 + q);
            r[4 * q + 0] = v.x;
            r[4 * q + 1] = v.y;
            r[4 * q + 2] = v.z;
            r[4 * q + 3] = v.w;
        }
    } else if constexpr (sizeof(T) == 8 && (C % 2) == 0) {
        const double2* s2 = reinterpret_cast<const double2*>(src + g0);
#pragma unroll
        for (int q = 0; q < C / 2; q++) {
            double2 v = CG ? __ldcg(s2 + q) : __ldcs(s2 + q);
            r[2 * q + 0] = v.x;
            r[2 * q + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < C; j++) r[j] = CG ? __ldcg(src + g0 + j) : __ldcs(src + g0 + j);
    }
}

template<typename T, int C>
__device__ __forceinline__ void store_cells(
    const T (&r)[C],
    T* __restrict__ dst,
    int64_t g0,
    int64_t l0,
    int64_t lo,
    int64_t hi)
{
    if (l0 >= lo && l0 + C <= hi) {
        if constexpr (sizeof(T) == 4 && (C % 4) == 0) {
            float4* d4 = reinterpret_cast<float4*>(dst + g0);
#pragma unroll
            for (int q = 0; q < C / 4; q++)
                __stcs(d4 + q, make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]));
            return;
        } else if constexpr (sizeof(T) == 8 && (C % 2) == 0) {
            double2* d2 = reinterpret_cast<double2*>(dst + g0);
#pragma unroll
            for (int q = 0; q < C / 2; q++) __stcs(d2 + q, make_double2(r[2 * q], r[2 * q + 1]));
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < C; j++)
        if (l0 + j >= lo && l0 + j < hi) dst[g0 + j] = r[j];
}

// An opaque copy of a pointer: loads through it can neither be hoisted out
// of the time loop nor shared between the two passes of one step. For 4 and
// more levels the compiler would otherwise keep the V x V coefficients live
// across steps and spill them to local memory.
template<typename T>
__device__ __forceinline__ const T* opaque_ptr(const T* p)
{
    const T* r;
    asm volatile("mov.b64 %0, %1;" : "=l"(r) : "l"(p));
    return r;
}

// Coefficients of the coherence-vector update, read through a pointer
// (shared memory for uniform tiles, global memory otherwise).
template<typename T, int V>
struct cvr_coef {
    static constexpr bool VEC = false;
    static constexpr int KP = V / 2;
    static constexpr int oBd = pre::FDTD_END;
    static constexpr int oBdl = oBd + V * V;
    static constexpr int ok = oBdl + V * V;
    static constexpr int og = ok + V;
    static constexpr int oth = og + V;
    const T* base;
    __device__ __forceinline__ T Bd(int i, int j) const { return base[oBd + i * V + j]; }
    __device__ __forceinline__ T Bdl(int i, int j) const { return base[oBdl + i * V + j]; }
    __device__ __forceinline__ T k(int i) const { return base[ok + i]; }
    __device__ __forceinline__ T g(int i) const { return base[og + i]; }
    __device__ __forceinline__ T th(int k) const { return base[oth + k]; }
    __device__ __forceinline__ T p0() const { return base[5]; }
    // the coefficients of one pass (see opaque_ptr)
    __device__ __forceinline__ cvr_coef pass() const
    {
        if constexpr (V >= 15)
            return cvr_coef{ opaque_ptr(base) };
        else
            return *this;
    }
};

// Compile-time loop: f(integral_constant<int, i>) for i in [B, E). Keeps
// every array index a constant so per-point vectors stay in registers
// (plain unrolled nested loops of 35 x 35 are not always fully unrolled).
template<int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f)
{
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// Shared-memory copy of a material's coherence-vector coefficients for 4 and
// more levels (V >= 15): the rows of Bd and Bdl are padded with zeros to a
// multiple of 16 bytes so that the updates read them with 128-bit loads
// (with scalar loads the 35 x 35 products of 6 levels are bound by the
// shared-memory load rate, one load per FMA). k, g and theta dt follow
// unchanged; the FDTD head (indices < FDTD_END, p0 at 5) is the same.
template<typename T, int V>
struct cvr_pad {
    static constexpr int W = 16 / (int) sizeof(T);  // reals per 16 bytes
    static constexpr int VP = (V + W - 1) / W * W;
    static constexpr int KP = V / 2;
    static constexpr int oBd = pre::FDTD_END;       // 48 or 96 bytes: aligned
    static constexpr int oBdl = oBd + V * VP;
    static constexpr int ok = oBdl + V * VP;
    static constexpr int og = ok + V;
    static constexpr int oth = og + V;
    static constexpr int len = oth + (KP > 0 ? KP : 1);
    // index in the material block for index i of the padded copy, -1: zero
    __device__ __forceinline__ static int source(int i)
    {
        const int bd = pre::FDTD_END, bdl = bd + V * V, k = bdl + V * V;
        if (i < oBd) return i;
        if (i < ok) {
            const int t = i < oBdl ? i - oBd : i - oBdl;
            const int r = t / VP, c = t % VP;
            if (c >= V) return -1;
            return (i < oBdl ? bd : bdl) + r * V + c;
        }
        return k + (i - ok);
    }
};

// 16 bytes of shared memory at a shared-window address
__device__ __forceinline__ void lds16(uint32_t a, float (&v)[4])
{
    asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
        : "r"(a));
}
__device__ __forceinline__ void lds16(uint32_t a, double (&v)[2])
{
    asm("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v[0]), "=d"(v[1]) : "r"(a));
}

// Accessor of the padded copy. Loads go through a shared-window address that
// is made opaque once per pass (see opaque_ptr).
template<typename T, int V>
struct cvr_coef_pad {
    using Lp = cvr_pad<T, V>;
    static constexpr bool VEC = true;
    static constexpr int W = Lp::W;
    uint32_t sbase;  // shared-window address of the copy
    const T* base;
    __device__ __forceinline__ T k(int i) const { return base[Lp::ok + i]; }
    __device__ __forceinline__ T g(int i) const { return base[Lp::og + i]; }
    __device__ __forceinline__ T th(int q) const { return base[Lp::oth + q]; }
    __device__ __forceinline__ T p0() const { return base[5]; }
    // W consecutive entries of row i of Bd (Bdl), from column W q
    __device__ __forceinline__ void Bdv(int i, int q, T (&v)[W]) const
    {
        lds16(sbase + (uint32_t) ((Lp::oBd + i * Lp::VP + W * q) * (int) sizeof(T)), v);
    }
    __device__ __forceinline__ void Bdlv(int i, int q, T (&v)[W]) const
    {
        lds16(sbase + (uint32_t) ((Lp::oBdl + i * Lp::VP + W * q) * (int) sizeof(T)), v);
    }
    __device__ __forceinline__ cvr_coef_pad pass() const
    {
        uint32_t a;
        asm volatile("mov.b32 %0, %1;" : "=r"(a) : "r"(sbase));
        return cvr_coef_pad{ a, opaque_ptr(base) };
    }
};

// s + sum_j Bd(I, j) x[j] (and sl + sum_j Bdl(I, j) x[j] when LO), with
// vector loads where the accessor has them
template<bool LO, int I, typename T, int V, class CF>
__device__ __forceinline__ void row_dot(const CF& c, const T (&x)[V], T& s, T& sl)
{
    if constexpr (CF::VEC) {
        constexpr int W = CF::W;
        static_for<0, (V + W - 1) / W>([&](auto Q) {
            constexpr int q = decltype(Q)::value;
            T b[W], bl[W];
            c.Bdv(I, q, b);
            if constexpr (LO) c.Bdlv(I, q, bl);
            static_for<0, W>([&](auto R) {
                constexpr int r = decltype(R)::value;
                constexpr int j = W * q + r;
                if constexpr (j < V) {
                    s = fma(b[r], x[j], s);
                    if constexpr (LO) sl = fma(bl[r], x[j], sl);
                }
            });
        });
    } else {
        static_for<0, V>([&](auto J) {
            constexpr int j = decltype(J)::value;
            s = fma(c.Bd(I, j), x[j], s);
            if constexpr (LO) sl = fma(c.Bdl(I, j), x[j], sl);
        });
    }
}

// Coherence-vector step in the plane basis, on the state v kept one half
// step ahead (see cvr_layout in precompute.cuh): rotate each plane by
// theta_k dt e; v = v + (Bd v + k); P = p0 + g . v.
template<typename T, int V, class CF>
__device__ __forceinline__ void cvr_update(T (&u)[V], T e, T& pout, const CF& cf)
{
    const auto c = cf.pass();
    static_for<0, V / 2>([&](auto K) {
        constexpr int k = decltype(K)::value;
        T sn, s2;
        rot_coeffs<T>(c.th(k) * e, sn, s2);
        T a = u[2 * k], b = u[2 * k + 1];
        u[2 * k] = a - fma(s2, a, sn * b);
        u[2 * k + 1] = b + fma(sn, a, -s2 * b);
    });
    T s[V];
    static_for<0, V>([&](auto I) {
        constexpr int i = decltype(I)::value;
        T sl = T(0);
        s[i] = c.k(i);
        row_dot<false, i>(c, u, s[i], sl);
    });
    T pp = c.p0();
    static_for<0, V>([&](auto I) {
        constexpr int i = decltype(I)::value;
        u[i] += s[i];
        pp = fma(c.g(i), u[i], pp);
    });
    pout = pp;
}

// hi + lo <- hi + lo + d, TwoSum without renormalising: lo collects the
// exact rounding error of the high word (and extra_lo)
__device__ __forceinline__ void df_acc(float& h, float& l, float d, float extra_lo)
{
    const float s = h + d;
    const float bv = s - h;
    const float err = (h - (s - bv)) + (d - bv);
    h = s;
    l = l + (err + extra_lo);
}

// renormalise a pair so that |lo| <= ulp(hi)/2 (Fast2Sum)
__device__ __forceinline__ void df_renorm(float& h, float& l)
{
    const float s = h + l;
    l = l - (s - h);
    h = s;
}

// Coefficients of the 2-level update held in registers (uniform tiles).
template<typename T, int V>
struct cvr_coef_reg {
    static constexpr bool VEC = false;
    T bd[V * V], bdl[V * V], kk[V], gg[V], thv[V / 2 > 0 ? V / 2 : 1], pz;
    __device__ __forceinline__ explicit cvr_coef_reg(const T* base)
    {
        cvr_coef<T, V> c{ base };
#pragma unroll
        for (int i = 0; i < V; i++) {
#pragma unroll
            for (int j = 0; j < V; j++) {
                bd[i * V + j] = c.Bd(i, j);
                bdl[i * V + j] = c.Bdl(i, j);
            }
            kk[i] = c.k(i);
            gg[i] = c.g(i);
        }
#pragma unroll
        for (int q = 0; q < V / 2; q++) thv[q] = c.th(q);
        pz = c.p0();
    }
    __device__ __forceinline__ T Bd(int i, int j) const { return bd[i * V + j]; }
    __device__ __forceinline__ T Bdl(int i, int j) const { return bdl[i * V + j]; }
    __device__ __forceinline__ T k(int i) const { return kk[i]; }
    __device__ __forceinline__ T g(int i) const { return gg[i]; }
    __device__ __forceinline__ T th(int q) const { return thv[q]; }
    __device__ __forceinline__ T p0() const { return pz; }
    __device__ __forceinline__ const cvr_coef_reg& pass() const { return *this; }  // stays in registers
};

// The same step in FP32 with v = uh + ul: the rotation increment d and
// the correction s = k + Bd r, r = fl(uh + d) the rotated high words, are
// computed in FP32 and their sum d + s is accumulated error-free (one
// TwoSum per entry; rounding d + s first costs ~3e-8 of an increment of
// ~1e-2, far below the low words' resolution); the low words take the
// rounding errors and the Bdl contribution; one renormalisation per step.
template<int V, class CF>
__device__ __forceinline__ void cvr_update_df(float (&uh)[V], float (&ul)[V], float e, float& pout, const CF& cf)
{
    const auto c = cf.pass();
    float d[V], r[V];
    static_for<0, V>([&](auto I) {
        constexpr int i = decltype(I)::value;
        d[i] = 0.0f;
        r[i] = uh[i];
    });
    static_for<0, V / 2>([&](auto K) {
        constexpr int k = decltype(K)::value;
        float sn, s2;
        rot_coeffs<float>(c.th(k) * e, sn, s2);
        const float a = r[2 * k], b = r[2 * k + 1];
        d[2 * k] = -fmaf(s2, a, sn * b);
        d[2 * k + 1] = fmaf(sn, a, -s2 * b);
        r[2 * k] = a + d[2 * k];
        r[2 * k + 1] = b + d[2 * k + 1];
    });
    float s[V], sl[V];
    static_for<0, V>([&](auto I) {
        constexpr int i = decltype(I)::value;
        s[i] = c.k(i);
        sl[i] = 0.0f;
        row_dot<true, i>(c, r, s[i], sl[i]);
    });
    float pp = c.p0();
    static_for<0, V>([&](auto I) {
        constexpr int i = decltype(I)::value;
        df_acc(uh[i], ul[i], d[i] + s[i], sl[i]);
        df_renorm(uh[i], ul[i]);
        pp = fmaf(c.g(i), uh[i], fmaf(c.g(i), ul[i], pp));
    });
    pout = pp;
}

// Value of a record at one point (solver_cpu_fdtd.tpp:301-325), on the
// kernels' state z (the coherence vector half a step ahead, see
// cvr_layout); REC_COH_RE / REC_COH_IM: the parts of a coherence record
// (no reference counterpart).
template<typename T, int V>
__device__ __forceinline__ T cvr_record_value(
    const rec_desc& rc,
    T e,
    T h,
    T pt,
    const T (&z)[V > 0 ? V : 1],
    const T* mcb,
    int N)
{
    switch (rc.type) {
    case 0:
        return e;
    case 1:
        return pt;
    case 2:
        return h;
    }
    if constexpr (V == 0) {
        return T(0);
    } else {
        // inversion, population and coherence parts: one row of the
        // material block on the state (inv, pop, coh in cvr_layout)
        pre::cvr_layout L = pre::make_cvr_layout(N);
        int row, c;
        if (rc.type == 4) {  // inversion d[N(N-1)]
            row = L.inv;
            c = L.inv_c;
        } else if (rc.type == 3) {
            if (rc.row_idx != rc.col_idx) return T(0);  // coherences: left zero
            int m = (int) rc.row_idx;
            // out-of-range level: what cvr.hpp:289-336 returns for it
            if (m >= N) {
                if (N == 2)
                    m = 1;
                else
                    return (N == 3) ? T(0) : T(1.0 / N);
            }
            row = L.pop + m * V;
            c = L.pop_c + m;
        } else {  // REC_COH_RE / REC_COH_IM: rho[a][b], a < b, pair q
            const int a = (int) min(rc.row_idx, rc.col_idx), b = (int) max(rc.row_idx, rc.col_idx);
            const int r = 2 * (b * (b - 1) / 2 + a) + (rc.type == REC_COH_IM ? 1 : 0);
            row = L.coh + r * V;
            c = L.coh_c + r;
        }
        T s = mcb[c];
#pragma unroll
        for (int k = 0; k < V; k++) s += mcb[row + k] * z[k];
        // rho[b][a] is the conjugate of rho[a][b]
        return (rc.type == REC_COH_IM && rc.row_idx > rc.col_idx) ? -s : s;
    }
}

// ------------------------------------------------------- field updates

struct fcoef {
    float a, bh, bl, g, ch, cl;
};

__device__ __forceinline__ fcoef load_fcoef(const float* cb)
{
    return fcoef{ cb[pre::FD_A], cb[pre::FD_BDX], cb[pre::FD_BDX_LO],
                  cb[pre::FD_G], cb[pre::FD_C], cb[pre::FD_C_LO] };
}

// hi + lo <- a (hi + lo) + (b/dx) (dh + dl) - b Gamma P, error-free except
// for the final renormalisation
__device__ __forceinline__ void df_e_update(
    float& eh,
    float& el,
    float dh,
    float dl,
    float pt,
    const fcoef& f)
{
    const float ph = f.bh * dh;
    const float pe = fmaf(f.bh, dh, -ph);
    const float pl = pe + fmaf(f.bh, dl, f.bl * dh) - f.g * pt;
    float xh = eh, xl = el;
    if (f.a != 1.0f) {
        xh = f.a * eh;
        xl = fmaf(f.a, eh, -xh) + f.a * el;
    }
    const float s = xh + ph;
    const float bv = s - xh;
    const float err = (xh - (s - bv)) + (ph - bv);
    const float e2 = err + (xl + pl);
    eh = s + e2;
    el = e2 - (eh - s);
}

// hi + lo <- hi + lo + c (dh + dl)
__device__ __forceinline__ void df_h_update(float& hh, float& hl, float dh, float dl, const fcoef& f)
{
    const float ph = f.ch * dh;
    const float pe = fmaf(f.ch, dh, -ph);
    const float pl = pe + fmaf(f.ch, dl, f.cl * dh);
    const float s = hh + ph;
    const float bv = s - hh;
    const float err = (hh - (s - bv)) + (ph - bv);
    const float e2 = err + (hl + pl);
    hh = s + e2;
    hl = e2 - (hh - s);
}

// hi + lo += v (v in FP64)
__device__ __forceinline__ void df_add(float& hh, float& hl, double v)
{
    const float vh = (float) v;
    const float vl = (float) (v - (double) vh);
    const float s = hh + vh;
    const float bv = s - hh;
    const float err = (hh - (s - bv)) + (vh - bv);
    const float e2 = err + (hl + vl);
    hh = s + e2;
    hl = e2 - (hh - s);
}

// ---------------------------------------------------- Cayley kernel
//
// Density matrix per point packed as N real populations followed by the
// upper off-diagonal triangle (column-major) as (re, im) pairs. One step of
// lindblad_reg_cayley::update (algo_lindblad_reg_cayley.hpp:228-257):
//   rho1 = D(rho); rho2 = U2 rho1 U2^H; rho = D(rho2);
//   P = n Re tr((-i/hbar [H0, rho] + D'(rho)) mu)
// with U2 = (I - m/2)^-1 (I + m/2), m = -i dt/hbar (H0 - e mu). Writing
// K = kappa (H0 - e mu), kappa = dt/(2 hbar): U2 = I + X with
// X = -2i (I + iK)^-1 K, so rho2 = rho1 + X rho1 + (X rho1)^H + X rho1 X^H,
// every term a small correction (accurate in FP32). D adds (D1 - I) and
// (D2 - 1) corrections.

struct cpx_f {
    float re, im;
};
struct cpx_d {
    double re, im;
};
template<typename T>
struct cpx_t;
template<>
struct cpx_t<float> {
    typedef cpx_f type;
};
template<>
struct cpx_t<double> {
    typedef cpx_d type;
};

template<typename T, int N>
__device__ __forceinline__ void cayley_update(T (&rho)[N * N], T e, T& pout, const T* cf)
{
    typedef typename cpx_t<T>::type cx;
    constexpr int P = N * (N - 1) / 2;
    const pre::cay_layout L = pre::make_cay_layout(N);
    // full K (Hermitian), A = I + i K
    cx K[N][N], A[N][N], Y[N][N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        K[i][i].re = cf[L.kH0 + i] - e * cf[L.kMu + i];
        K[i][i].im = T(0);
    }
#pragma unroll
    for (int k = 1; k < N; k++)
#pragma unroll
        for (int j = 0; j < k; j++) {
            const int q = k * (k - 1) / 2 + j;
            T re = cf[L.kH0 + N + 2 * q] - e * cf[L.kMu + N + 2 * q];
            T im = cf[L.kH0 + N + 2 * q + 1] - e * cf[L.kMu + N + 2 * q + 1];
            K[j][k].re = re;
            K[j][k].im = im;
            K[k][j].re = re;
            K[k][j].im = -im;
        }
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) {
            // i K = (-K.im, K.re)
            A[i][j].re = -K[i][j].im + (i == j ? T(1) : T(0));
            A[i][j].im = K[i][j].re;
            Y[i][j] = K[i][j];
        }
    // solve A Y = K by LU without pivoting (A + A^H = 2I > 0); the inverse
    // of each pivot (one real division) serves elimination and
    // back-substitution (a pivot is final once its step begins)
    cx pinv[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        const T rden = T(1) / (A[k][k].re * A[k][k].re + A[k][k].im * A[k][k].im);
        cx inv;
        inv.re = A[k][k].re * rden;
        inv.im = -A[k][k].im * rden;
        pinv[k] = inv;
#pragma unroll
        for (int i = k + 1; i < N; i++) {
            cx f;
            f.re = A[i][k].re * inv.re - A[i][k].im * inv.im;
            f.im = A[i][k].re * inv.im + A[i][k].im * inv.re;
#pragma unroll
            for (int j = k + 1; j < N; j++) {
                A[i][j].re -= f.re * A[k][j].re - f.im * A[k][j].im;
                A[i][j].im -= f.re * A[k][j].im + f.im * A[k][j].re;
            }
#pragma unroll
            for (int j = 0; j < N; j++) {
                Y[i][j].re -= f.re * Y[k][j].re - f.im * Y[k][j].im;
                Y[i][j].im -= f.re * Y[k][j].im + f.im * Y[k][j].re;
            }
        }
    }
#pragma unroll
    for (int k = N - 1; k >= 0; k--) {
        const cx inv = pinv[k];
#pragma unroll
        for (int j = 0; j < N; j++) {
            cx s = Y[k][j];
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                s.re -= A[k][i].re * Y[i][j].re - A[k][i].im * Y[i][j].im;
                s.im -= A[k][i].re * Y[i][j].im + A[k][i].im * Y[i][j].re;
            }
            Y[k][j].re = s.re * inv.re - s.im * inv.im;
            Y[k][j].im = s.re * inv.im + s.im * inv.re;
        }
    }
    // X = -2i Y  -> (2 Y.im, -2 Y.re); reuse K for X
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) {
            K[i][j].re = T(2) * Y[i][j].im;
            K[i][j].im = T(-2) * Y[i][j].re;
        }
    // rho1 = D(rho): full Hermitian R in A
    auto dissipate = [&](const T (&in)[N * N], cx (&R)[N][N]) {
#pragma unroll
        for (int i = 0; i < N; i++) {
            T s = in[i];
#pragma unroll
            for (int j = 0; j < N; j++) s = fma(cf[L.dD1 + i * N + j], in[j], s);
            R[i][i].re = s;
            R[i][i].im = T(0);
        }
#pragma unroll
        for (int k = 1; k < N; k++)
#pragma unroll
            for (int j = 0; j < k; j++) {
                const int q = k * (k - 1) / 2 + j;
                const T dd = cf[L.dD2 + q];
                T re = in[N + 2 * q], im = in[N + 2 * q + 1];
                re = fma(dd, re, re);
                im = fma(dd, im, im);
                R[j][k].re = re;
                R[j][k].im = im;
                R[k][j].re = re;
                R[k][j].im = -im;
            }
    };
    dissipate(rho, A);
    // G = X rho1 (in Y)
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) {
            cx s;
            s.re = T(0);
            s.im = T(0);
#pragma unroll
            for (int l = 0; l < N; l++) {
                s.re += K[i][l].re * A[l][j].re - K[i][l].im * A[l][j].im;
                s.im += K[i][l].re * A[l][j].im + K[i][l].im * A[l][j].re;
            }
            Y[i][j] = s;
        }
    // rho2 (packed) = rho1 + G + G^H + G X^H
    T r2[N * N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        T s = A[i][i].re + T(2) * Y[i][i].re;
#pragma unroll
        for (int l = 0; l < N; l++) s += Y[i][l].re * K[i][l].re + Y[i][l].im * K[i][l].im;
        r2[i] = s;
    }
#pragma unroll
    for (int k = 1; k < N; k++)
#pragma unroll
        for (int j = 0; j < k; j++) {
            const int q = k * (k - 1) / 2 + j;
            T re = A[j][k].re + Y[j][k].re + Y[k][j].re;
            T im = A[j][k].im + Y[j][k].im - Y[k][j].im;
#pragma unroll
            for (int l = 0; l < N; l++) {
                // G_jl conj(X_kl)
                re += Y[j][l].re * K[k][l].re + Y[j][l].im * K[k][l].im;
                im += Y[j][l].im * K[k][l].re - Y[j][l].re * K[k][l].im;
            }
            r2[N + 2 * q] = re;
            r2[N + 2 * q + 1] = im;
        }
    // rho = D(rho2), full matrix in A, packed into rho
    dissipate(r2, A);
#pragma unroll
    for (int i = 0; i < N; i++) rho[i] = A[i][i].re;
#pragma unroll
    for (int k = 1; k < N; k++)
#pragma unroll
        for (int j = 0; j < k; j++) {
            const int q = k * (k - 1) / 2 + j;
            rho[N + 2 * q] = A[j][k].re;
            rho[N + 2 * q + 1] = A[j][k].im;
        }
    // P = Re tr((-i [W0, rho] + D'(rho)) Mn), linear in the packed density
    // matrix: P = gP . rho (weights from the FP64 precompute)
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < N * N; i++) acc = fma(cf[L.gP + i], rho[i], acc);
    pout = acc;
}

// The same step in FP32 on rho = rh + rl (float pairs), split as in
// cay_layout: rho <- rho + B0 rho + D(E(D rho)). The field-free part B0 rho
// uses B0 and its low part B0l (error-free accumulation into the pair);
// the field-dependent correction E is computed in FP32 from the high words:
//   s = D(rh);  A(e) Y = W (LU without pivoting: A's Hermitian part is I);
//   dU = 2 i e Y;  Z = dU s;  E = Z (U0 + dU)^H + U0 Z^H.
// One renormalisation of the pairs per step; P = gP . rho.
template<int N>
__device__ __forceinline__ void cayley_update_df(float (&rh)[N * N], float (&rl)[N * N], float e, float& pout, const float* cf)
{
    typedef cpx_f cx;
    constexpr int NN = N * N;
    const pre::cay_layout L = pre::make_cay_layout(N);
    // s = D(rh), packed like rho (entry (l, k) through sget)
    float sp[NN];
#pragma unroll
    for (int i = 0; i < N; i++) {
        float v = rh[i];
#pragma unroll
        for (int j = 0; j < N; j++) v = fmaf(cf[L.dD1 + i * N + j], rh[j], v);
        sp[i] = v;
    }
#pragma unroll
    for (int q = 0; q < (NN - N) / 2; q++) {
        const float dd = cf[L.dD2 + q];
        sp[N + 2 * q] = fmaf(dd, rh[N + 2 * q], rh[N + 2 * q]);
        sp[N + 2 * q + 1] = fmaf(dd, rh[N + 2 * q + 1], rh[N + 2 * q + 1]);
    }
    auto sget = [&](int l, int k) -> cx {
        cx v;
        if (l == k) {
            v.re = sp[l];
            v.im = 0.0f;
        } else {
            const int a = l < k ? l : k, b = l < k ? k : l;
            const int q = b * (b - 1) / 2 + a;
            v.re = sp[N + 2 * q];
            v.im = l < k ? sp[N + 2 * q + 1] : -sp[N + 2 * q + 1];
        }
        return v;
    };
    // A = I + i (kappa H0 - e kappa mu); Y = W
    cx A[N][N], Y[N][N];
#pragma unroll
    for (int j = 0; j < N; j++)
#pragma unroll
        for (int k = 0; k < N; k++) {
            float kr, ki;
            if (j == k) {
                kr = fmaf(-e, cf[L.kMu + j], cf[L.kH0 + j]);
                ki = 0.0f;
            } else {
                const int a = j < k ? j : k, b = j < k ? k : j;
                const int q = b * (b - 1) / 2 + a;
                kr = fmaf(-e, cf[L.kMu + N + 2 * q], cf[L.kH0 + N + 2 * q]);
                ki = fmaf(-e, cf[L.kMu + N + 2 * q + 1], cf[L.kH0 + N + 2 * q + 1]);
                if (j > k) ki = -ki;
            }
            A[j][k].re = (j == k ? 1.0f : 0.0f) - ki;
            A[j][k].im = kr;
            Y[j][k].re = cf[L.Wk + j * N + k];
            Y[j][k].im = cf[L.Wk + NN + j * N + k];
        }
    cx pinv[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        const float rden = 1.0f / (A[k][k].re * A[k][k].re + A[k][k].im * A[k][k].im);
        cx inv;
        inv.re = A[k][k].re * rden;
        inv.im = -A[k][k].im * rden;
        pinv[k] = inv;
#pragma unroll
        for (int i = k + 1; i < N; i++) {
            cx f;
            f.re = A[i][k].re * inv.re - A[i][k].im * inv.im;
            f.im = A[i][k].re * inv.im + A[i][k].im * inv.re;
#pragma unroll
            for (int j = k + 1; j < N; j++) {
                A[i][j].re -= f.re * A[k][j].re - f.im * A[k][j].im;
                A[i][j].im -= f.re * A[k][j].im + f.im * A[k][j].re;
            }
#pragma unroll
            for (int j = 0; j < N; j++) {
                Y[i][j].re -= f.re * Y[k][j].re - f.im * Y[k][j].im;
                Y[i][j].im -= f.re * Y[k][j].im + f.im * Y[k][j].re;
            }
        }
    }
#pragma unroll
    for (int k = N - 1; k >= 0; k--) {
        const cx inv = pinv[k];
#pragma unroll
        for (int j = 0; j < N; j++) {
            cx v = Y[k][j];
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                v.re -= A[k][i].re * Y[i][j].re - A[k][i].im * Y[i][j].im;
                v.im -= A[k][i].re * Y[i][j].im + A[k][i].im * Y[i][j].re;
            }
            Y[k][j].re = v.re * inv.re - v.im * inv.im;
            Y[k][j].im = v.re * inv.im + v.im * inv.re;
        }
    }
    // dU = 2 i e Y (in Y); Z = dU s (in A)
    const float e2 = 2.0f * e;
#pragma unroll
    for (int j = 0; j < N; j++)
#pragma unroll
        for (int k = 0; k < N; k++) {
            const float yr = Y[j][k].re;
            Y[j][k].re = -e2 * Y[j][k].im;
            Y[j][k].im = e2 * yr;
        }
#pragma unroll
    for (int j = 0; j < N; j++)
#pragma unroll
        for (int k = 0; k < N; k++) {
            float zr = 0.0f, zi = 0.0f;
#pragma unroll
            for (int l = 0; l < N; l++) {
                const cx s = sget(l, k);
                zr = fmaf(Y[j][l].re, s.re, fmaf(-Y[j][l].im, s.im, zr));
                zi = fmaf(Y[j][l].re, s.im, fmaf(Y[j][l].im, s.re, zi));
            }
            A[j][k].re = zr;
            A[j][k].im = zi;
        }
    // E (packed) = Z (U0 + dU)^H + U0 Z^H
    float ev[NN];
#pragma unroll
    for (int k = 0; k < N; k++)
#pragma unroll
        for (int j = 0; j <= k; j++) {
            float er = 0.0f, ei = 0.0f;
#pragma unroll
            for (int l = 0; l < N; l++) {
                const float u0r = cf[L.U0 + k * N + l], u0i = cf[L.U0 + NN + k * N + l];
                const float u2r = u0r + Y[k][l].re, u2i = u0i + Y[k][l].im;
                // Z_jl conj(U2_kl)
                er = fmaf(A[j][l].re, u2r, fmaf(A[j][l].im, u2i, er));
                ei = fmaf(A[j][l].im, u2r, fmaf(-A[j][l].re, u2i, ei));
                // U0_jl conj(Z_kl)
                const float v0r = cf[L.U0 + j * N + l], v0i = cf[L.U0 + NN + j * N + l];
                er = fmaf(v0r, A[k][l].re, fmaf(v0i, A[k][l].im, er));
                ei = fmaf(v0i, A[k][l].re, fmaf(-v0r, A[k][l].im, ei));
            }
            if (j == k) {
                ev[j] = er;
            } else {
                const int q = k * (k - 1) / 2 + j;
                ev[N + 2 * q] = er;
                ev[N + 2 * q + 1] = ei;
            }
        }
    // increments: D(E) + B0 rh (high part), B0l rh (low part)
    float inc[NN], incl[NN];
#pragma unroll
    for (int i = 0; i < N; i++) {
        float v = ev[i];
#pragma unroll
        for (int j = 0; j < N; j++) v = fmaf(cf[L.dD1 + i * N + j], ev[j], v);
        inc[i] = v;
    }
#pragma unroll
    for (int q = 0; q < (NN - N) / 2; q++) {
        const float dd = cf[L.dD2 + q];
        inc[N + 2 * q] = fmaf(dd, ev[N + 2 * q], ev[N + 2 * q]);
        inc[N + 2 * q + 1] = fmaf(dd, ev[N + 2 * q + 1], ev[N + 2 * q + 1]);
    }
    if (cf[L.blockB0] != 0.0f) {
        // diagonal H0: B0 is block-diagonal (populations; each coherence's
        // 2 x 2 block), the same sums without their exact zero terms
#pragma unroll
        for (int v = 0; v < NN; v++) {
            float a = inc[v], b = 0.0f;
            const int w0 = v < N ? 0 : N + ((v - N) & ~1), w1 = v < N ? N : w0 + 2;
#pragma unroll
            for (int w = w0; w < w1; w++) {
                a = fmaf(cf[L.B0 + v * L.NP + w], rh[w], a);
                b = fmaf(cf[L.B0l + v * L.NP + w], rh[w], b);
            }
            inc[v] = a;
            incl[v] = b;
        }
    } else {
#pragma unroll
        for (int v = 0; v < NN; v++) {
            float a = inc[v], b = 0.0f;
#pragma unroll
            for (int w = 0; w < NN; w++) {
                a = fmaf(cf[L.B0 + v * L.NP + w], rh[w], a);
                b = fmaf(cf[L.B0l + v * L.NP + w], rh[w], b);
            }
            inc[v] = a;
            incl[v] = b;
        }
    }
    float acc = 0.0f;
#pragma unroll
    for (int v = 0; v < NN; v++) {
        df_acc(rh[v], rl[v], inc[v], incl[v]);
        df_renorm(rh[v], rl[v]);
        acc = fmaf(cf[L.gP + v], rh[v], fmaf(cf[L.gP + v], rl[v], acc));
    }
    pout = acc;
}

}  // namespace mbg
