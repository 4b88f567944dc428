// The uniform-tile time loop of the 2-level FP32 kernel on packed FP32
// pairs (Blackwell's two-lane fma/add/mul/sub.rn.f32x2: one instruction
// updates two grid points, each lane rounded like the scalar operation).
//
// Point j of a thread shares a register pair with point j + C/2, so the
// right neighbour of pair q in the E update is pair q + 1 and the left
// neighbour in the H update pair q - 1; only the pair at the thread's edge
// is assembled from the neighbouring thread's value. Every operation is
// the one of tile_steps (the same products, sums and fused multiply-adds in
// the same order), so at every in-run point the results equal the scalar
// loop's. Threads whose points reach past a run end (point 0 or a point
// outside [0, n_x)) update every point like the others and then put the
// points that the scalar loop leaves alone back to their values there:
// H = 0 outside [1, n_x) (PMC at point 0, the zero state beyond the ends),
// and zero E, P and coherence vector outside [0, n_x).
#pragma once

#include "f32x2.cuh"
#include "kernels.cuh"

namespace mbg {

// The pair path runs for the CUDA-core 2-level FP32 kernels with an even
// number of points per thread.
template<typename T, int ALGO, int LEV, int C, bool TC>
constexpr bool pair_path()
{
    return sizeof(T) == 4 && ALGO == 1 && LEV == 2 && !TC && C % 2 == 0;
}

// The coefficients of a uniform tile, each broadcast to both lanes.
struct cvr2_pair_coef {
    float2 a, bh, mg, ch;  // E: a, b/dx, -b Gamma; H: c
    float2 th, p0, bd[9], bdl[9], k[3], g[3];
    __device__ __forceinline__ explicit cvr2_pair_coef(const float* cb)
    {
        const fcoef f = load_fcoef(cb);
        a = f2::bc(f.a);
        bh = f2::bc(f.bh);
        mg = f2::bc(-f.g);
        ch = f2::bc(f.ch);
        const cvr_coef<float, 3> c{ cb };
        th = f2::bc(c.th(0));
        p0 = f2::bc(c.p0());
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++) {
                bd[i * 3 + j] = f2::bc(c.Bd(i, j));
                bdl[i * 3 + j] = f2::bc(c.Bdl(i, j));
            }
            k[i] = f2::bc(c.k(i));
            g[i] = f2::bc(c.g(i));
        }
    }
};

// The couplings that the plane basis of a 2-level medium with a diagonal
// Hamiltonian and a real dipole leaves exactly zero: the field rotates the
// (0, 1) plane, the free evolution couples 0 and 2 (precession) and relaxes
// 1 on its own, and P reads 0 and 2. A uniform tile whose block has them
// zero skips their products (a product with an exact zero changes no sum).
__device__ __forceinline__ bool cvr2_sparse(const float* cb)
{
    const cvr_coef<float, 3> c{ cb };
    return c.Bd(0, 1) == 0.0f && c.Bd(1, 0) == 0.0f && c.Bd(1, 2) == 0.0f && c.Bd(2, 1) == 0.0f &&
        c.Bdl(0, 1) == 0.0f && c.Bdl(1, 0) == 0.0f && c.Bdl(1, 2) == 0.0f && c.Bdl(2, 1) == 0.0f &&
        c.g(1) == 0.0f;
}

// cvr_update_df<3> on two points: the rotation of the (0, 1) plane by
// theta dt e (rot_coeffs' series, its negated Horner chain for 1 - cos
// giving the same roundings), the correction k + Bd r with its low-word
// part Bdl r, the error-free accumulation and renormalisation of the pair
// words, and P = p0 + g . v. SP: the zeros of cvr2_sparse are skipped.
template<bool SP>
__device__ __forceinline__ void cvr2_update_pair(float2 (&uh)[3], float2 (&ul)[3], float2 e, float2& pout,
                                                 const cvr2_pair_coef& c)
{
    using namespace f2;
    const float2 z = bc(0.0f);
    const float2 x = mul(c.th, e);
    float2 sn, s2;
    if (fabsf(x.x) < 0.0078125f && fabsf(x.y) < 0.0078125f) {
        const float2 x2 = mul(x, x);
        sn = fma(mul(x, x2), bc(-1.0f / 6.0f), x);
        s2 = mul(x2, fma(x2, bc(-1.0f / 24.0f), bc(0.5f)));
    } else if (fabsf(x.x) < 0.0625f && fabsf(x.y) < 0.0625f) {
        const float2 x2 = mul(x, x);
        float2 t = fma(x2, bc(-1.0f / 5040.0f), bc(1.0f / 120.0f));
        t = fma(x2, t, bc(-1.0f / 6.0f));
        sn = fma(mul(x, x2), t, x);
        float2 v = fma(x2, bc(-1.0f / 40320.0f), bc(1.0f / 720.0f));
        v = fma(x2, v, bc(-1.0f / 24.0f));
        s2 = mul(x2, fma(x2, v, bc(0.5f)));
    } else {
        rot_coeffs<float>(x.x, sn.x, s2.x);
        rot_coeffs<float>(x.y, sn.y, s2.y);
    }
    const float2 a = uh[0], b = uh[1];
    // q0 = -d0; d1 = sn a - s2 b
    const float2 q0 = fma(s2, a, mul(sn, b));
    const float2 d1 = fma(sn, a, mul(sub(z, s2), b));
    const float2 r[3] = { sub(a, q0), add(b, d1), uh[2] };
    float2 s[3], sl[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        s[i] = c.k[i];
        sl[i] = z;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            if (SP && (i == 1) != (j == 1)) continue;
            s[i] = fma(c.bd[i * 3 + j], r[j], s[i]);
            sl[i] = fma(c.bdl[i * 3 + j], r[j], sl[i]);
        }
    }
    const float2 dd[3] = { sub(s[0], q0), add(d1, s[1]), s[2] };
    float2 pp = c.p0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float2 h = uh[i], l = ul[i];
        // TwoSum of h + dd, the error and Bdl r into the low word
        const float2 sum = add(h, dd[i]);
        const float2 bv = sub(sum, h);
        const float2 err = add(sub(h, sub(sum, bv)), sub(dd[i], bv));
        h = sum;
        l = add(l, add(err, sl[i]));
        // Fast2Sum renormalisation
        const float2 t = add(h, l);
        l = sub(l, sub(t, h));
        h = t;
        uh[i] = h;
        ul[i] = l;
        if (!SP || i != 1) pp = fma(c.g[i], h, fma(c.g[i], l, pp));
    }
    pout = pp;
}

template<int C>
struct pair_view {
    static constexpr int HP = C / 2;
    // point j of a thread: lane j / HP of pair j % HP
    __device__ __forceinline__ static float& at(float2 (&v)[HP], int j)
    {
        return j < HP ? v[j % HP].x : v[j % HP].y;
    }
    __device__ __forceinline__ static float& at3(float2 (&v)[HP][3], int j, int i)
    {
        return j < HP ? v[j % HP][i].x : v[j % HP][i].y;
    }
};

// TL: tile_lists (tile_kernel.cuh); SP: the tile's block has the zeros of
// cvr2_sparse
template<int C, int NT, bool SP, class TL>
__device__ __forceinline__ void tile_steps_pair(
    const kparams<float>& p,
    const tile_desc& td,
    const run_desc& rd,
    int64_t l0,
    int nsteps,
    uint64_t step0,
    float (&E)[C],
    float (&H)[C],
    float (&P)[C],
    float (&R)[C][3],
    float (&Rl)[C][3],
    const int32_t (&M)[C],
    const float* sh_coef,
    const TL& tl,
    float* sh_a,
    float* sh_b)
{
    using namespace f2;
    constexpr int HP = C / 2;
    constexpr int NW = NT / 32;
    using V = pair_view<C>;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t nx = rd.n_x;
    float2 e[HP], h[HP], pt[HP], u[HP][3], ul[HP][3];
#pragma unroll
    for (int q = 0; q < HP; q++) {
        e[q] = make_float2(E[q], E[q + HP]);
        h[q] = make_float2(H[q], H[q + HP]);
        pt[q] = make_float2(P[q], P[q + HP]);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            u[q][i] = make_float2(R[q][i], R[q + HP][i]);
            ul[q][i] = make_float2(Rl[q][i], Rl[q + HP][i]);
        }
    }
    const cvr2_pair_coef cf(sh_coef);
    const bool qm = sh_coef[pre::FD_HAS_QM] != 0.0f;
    // every point of the thread inside [1, n_x): no point to put back
    const bool interior = l0 >= 1 && l0 + C <= nx;
    const int nsrc = tl.overflow ? (int) (rd.src_end - rd.src_begin) : tl.nsrc;
    const int nrec = tl.overflow ? (int) (rd.rec_end - rd.rec_begin) : tl.nrec;
    for (int m = 0; m < nsteps; m++) {
        const uint64_t n = step0 + (uint64_t) m;
        // ---- E: needs H of the right neighbour
        if (lane == 0) sh_a[warp] = h[0].x;
        __syncthreads();
        float hr = __shfl_down_sync(0xffffffffu, h[0].x, 1);
        if (lane == 31) hr = (warp + 1 < NW) ? sh_a[warp + 1] : 0.0f;
#pragma unroll
        for (int q = 0; q < HP; q++) {
            const float2 hn = (q + 1 < HP) ? h[q + 1] : make_float2(h[0].y, hr);
            e[q] = fma(cf.a, e[q], fma(cf.bh, sub(hn, h[q]), mul(cf.mg, pt[q])));
        }
        // ---- sources, after E and before H (solver_cpu_fdtd.tpp:245-255)
        for (int s = 0; s < nsrc; s++) {
            const src_desc sd = tl.overflow ? p.srcs[rd.src_begin + s] : tl.src[s];
            const int64_t jj = (int64_t) sd.x_idx - l0;
            if (jj >= 0 && jj < C) {
                const double v = p.stab[sd.table_offset + n];
#pragma unroll
                for (int j = 0; j < C; j++) {
                    if (j != jj || M[j] < 0) continue;
                    if (sd.type == 0)
                        V::at(e, j) = (float) v;
                    else
                        V::at(e, j) += (float) v;
                }
            }
        }
        // ---- H: needs E of the left neighbour
        if (lane == 31) sh_b[warp] = e[HP - 1].y;
        __syncthreads();
        float el = __shfl_up_sync(0xffffffffu, e[HP - 1].y, 1);
        if (lane == 0) el = (warp > 0) ? sh_b[warp - 1] : 0.0f;
#pragma unroll
        for (int q = 0; q < HP; q++) {
            const float2 ep = (q > 0) ? e[q - 1] : make_float2(el, e[HP - 1].x);
            h[q] = fma(cf.ch, sub(e[q], ep), h[q]);
        }
        if (!interior) {
#pragma unroll
            for (int j = 0; j < C; j++) {
                const int64_t l = l0 + j;
                if (l < 1 || l >= nx) V::at(h, j) = 0.0f;  // PMC (solver_cpu_fdtd.tpp:273)
            }
        }
        // ---- coherence vector and polarisation at every point
        if (qm) {
#pragma unroll
            for (int q = 0; q < HP; q++) cvr2_update_pair<SP>(u[q], ul[q], e[q], pt[q], cf);
        }
        if (!interior) {
#pragma unroll
            for (int j = 0; j < C; j++) {
                if (M[j] >= 0) continue;
                V::at(e, j) = V::at(pt, j) = 0.0f;
#pragma unroll
                for (int i = 0; i < 3; i++) V::at3(u, j, i) = V::at3(ul, j, i) = 0.0f;
            }
        }
        // ---- recording (solver_cpu_fdtd.tpp:288-325)
        if (p.record) {
            for (int r = 0; r < nrec; r++) {
                const rec_desc rc = tl.overflow ? p.recs[rd.rec_begin + r] : tl.rec[r];
                if (rc.ratio != 1.0 && !hasto_record(rc.ratio, n)) continue;
                const int64_t lo = max((int64_t) rc.pos, (int64_t) td.out_start);
                const int64_t hi = min((int64_t) rc.pos + rc.cols, (int64_t) td.out_start + td.out_len);
                if (l0 + C <= lo || l0 >= hi) continue;
                const uint64_t row = rc.ratio == 1.0 ? n : (uint64_t) floor(rc.ratio * (double) n);
                if (row >= rc.rows) continue;
#pragma unroll
                for (int j = 0; j < C; j++) {
                    const int64_t l = l0 + j;
                    if (l < lo || l >= hi) continue;
                    float w[3];
#pragma unroll
                    for (int i = 0; i < 3; i++) w[i] = V::at3(u, j, i) + V::at3(ul, j, i);
                    // the coherence rows are not staged in shared memory
                    const float* rb = rc.type >= REC_COH_RE ? p.mc + (uint64_t) M[j] * p.mstride : sh_coef;
                    const float v = cvr_record_value<float, 3>(rc, V::at(e, j), V::at(h, j), V::at(pt, j), w, rb, 2);
                    p.scratch[rc.offset + row * rc.cols + (uint64_t) (l - rc.pos)] = v;
                    if (!isfinite(v)) atomicOr(p.status, STATUS_NONFINITE);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < HP; q++) {
        E[q] = e[q].x;
        E[q + HP] = e[q].y;
        H[q] = h[q].x;
        H[q + HP] = h[q].y;
        P[q] = pt[q].x;
        P[q + HP] = pt[q].y;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            R[q][i] = u[q][i].x;
            R[q + HP][i] = u[q][i].y;
            Rl[q][i] = ul[q][i].x;
            Rl[q + HP][i] = ul[q][i].y;
        }
    }
}

}  // namespace mbg
