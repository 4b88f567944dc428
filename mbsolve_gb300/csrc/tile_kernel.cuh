// The tile kernel: one launch advances every tile of every run by up to
// `nsub` time steps (see kernels.cuh for the scheme and the per-point
// updates).
//
// ALGO 0: Maxwell only (algo_lindblad_noop.hpp), 1: coherence vector /
// Rodrigues, 2: Cayley. D density reals per point: 0, N^2 - 1, N^2.
#pragma once

#include <type_traits>

#include "kernels.cuh"
#include "tc_density.cuh"
#include "bulk_stage.cuh"
#include "pair_steps.cuh"

namespace mbg {

template<int ALGO, int LEV>
struct density_len {
    static constexpr int value = ALGO == 1 ? LEV * LEV - 1 : ALGO == 2 ? LEV * LEV : 0;
};

// sources and records that touch one tile, gathered once per launch
constexpr int TILE_MAX_SRC = 8;
constexpr int TILE_MAX_REC = 8;

struct no_coef {
    __device__ __forceinline__ explicit no_coef(const void*) {}
};

struct tile_lists {
    int nsrc, nrec, overflow;
    int wall;  // the window holds a mirror wall (run_desc k_left, k_right)
    src_desc src[TILE_MAX_SRC];
    rec_desc rec[TILE_MAX_REC];
};

// Returns false when a tensor-core wait ran out (TC kernels only).
template<typename T, int ALGO, int LEV, int C, int NT, bool UNIFORM, bool TC = false>
__device__ __forceinline__ bool tile_steps(
    const kparams<T>& p,
    const tile_desc& td,
    const run_desc& rd,
    int64_t l0,
    int nsteps,
    uint64_t step0,
    T (&E)[C],
    T (&El)[C],
    T (&H)[C],
    T (&Hl)[C],
    T (&P)[C],
    T (&R)[C][density_len<ALGO, LEV>::value > 0 ? density_len<ALGO, LEV>::value : 1],
    T (&Rl)[C][density_len<ALGO, LEV>::value > 0 ? density_len<ALGO, LEV>::value : 1],
    const int32_t (&M)[C],
    const T* sh_coef,
    const tile_lists& tl,
    T* sh_a,
    T* sh_al,
    T* sh_b,
    T* sh_bl,
    tc::ctx* tcc = nullptr)
{
    // FP32: the density state is a float pair (hi + lo) throughout; E and H
    // are float pairs except in the 2-level coherence-vector kernel, where
    // plain FP32 fields (one rounding per update, coefficients in
    // registers) hold the probe error near 6e-6 at 100,000 steps, under
    // the 1e-5 target, at 22 % more cell-updates/s (measured variant by
    // variant: a plain FP32 coherence vector instead broke 1e-5)
    constexpr bool DFD = sizeof(T) == 4;
    constexpr bool DF = DFD && !(ALGO == 1 && LEV == 2);
    constexpr int D = density_len<ALGO, LEV>::value;
    constexpr int NW = NT / 32;
    constexpr bool TCU = TC && UNIFORM;  // density products on the tensor cores
    static_assert(!TC || (DF && ALGO == 1 && D >= 15 && C == 1 && NT == tc::M), "TC kernel shape");
    // 2-level coefficients live in registers on uniform tiles; for 4 and more
    // levels uniform tiles hold the padded copy of cvr_pad in shared memory
    constexpr bool REGCOEF = UNIFORM && ALGO == 1 && D == 3;
    constexpr bool PADC = UNIFORM && ALGO == 1 && D >= 15;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t nx = rd.n_x;
    const T dxi = (T) rd.dx_inv;
    auto block = [&](int j) -> const T* {
        return UNIFORM ? sh_coef : p.mc + (uint64_t) (M[j] >= 0 ? M[j] : 0) * p.mstride;
    };
    fcoef fu;
    if constexpr (DFD && UNIFORM) fu = load_fcoef(sh_coef);
    const bool qm_uniform = UNIFORM && sh_coef[pre::FD_HAS_QM] != T(0);
    using creg_t = typename std::conditional<REGCOEF, cvr_coef_reg<T, 3>, no_coef>::type;
    const creg_t creg(sh_coef);
    const int nsrc = tl.overflow ? (int) (rd.src_end - rd.src_begin) : tl.nsrc;
    const int nrec = tl.overflow ? (int) (rd.rec_end - rd.rec_begin) : tl.nrec;
    // Mirror walls are handled only on tiles of the non-uniform path (the
    // set-up marks a tile whose window holds a wall non-uniform): code that
    // touches H around the time loop, even off its hot path, costs the
    // uniform 2-level kernel 5-8 % (measured).
    if (!UNIFORM && tl.wall && rd.k_right != 0.0) {
        // mirror: the point beyond the right end loads as zero state; give
        // it its wall value -k_right E[nx - 1] before the first step (the H
        // update keeps it from then on). rd is the same in the whole CTA.
        if (lane == 31) {
            sh_b[warp] = E[C - 1];
            if constexpr (DF) sh_bl[warp] = El[C - 1];
        }
        __syncthreads();
        T el = __shfl_up_sync(0xffffffffu, E[C - 1], 1);
        T ell = DF ? __shfl_up_sync(0xffffffffu, El[C - 1], 1) : T(0);
        if (lane == 0) {
            el = (warp > 0) ? sh_b[warp - 1] : T(0);
            if constexpr (DF) ell = (warp > 0) ? sh_bl[warp - 1] : T(0);
        }
        const T k_right = (T) rd.k_right;
#pragma unroll
        for (int j = 0; j < C; j++)
            if (l0 + j == nx) {
                H[j] = -k_right * ((j > 0) ? E[j - 1] : el);
                if constexpr (DF) Hl[j] = -k_right * ((j > 0) ? El[j - 1] : ell);
            }
        // sh_b is written again only after the next barrier (E phase)
    }
    for (int m = 0; m < nsteps; m++) {
        const uint64_t n = step0 + (uint64_t) m;
        // ---- E: needs H (hi, lo) of the right neighbour
        if (lane == 0) {
            sh_a[warp] = H[0];
            if constexpr (DF) sh_al[warp] = Hl[0];
        }
        __syncthreads();
        T hr = __shfl_down_sync(0xffffffffu, H[0], 1);
        T hrl = DF ? __shfl_down_sync(0xffffffffu, Hl[0], 1) : T(0);
        if (lane == 31) {
            hr = (warp + 1 < NW) ? sh_a[warp + 1] : T(0);
            if constexpr (DF) hrl = (warp + 1 < NW) ? sh_al[warp + 1] : T(0);
        }
#pragma unroll
        for (int j = 0; j < C; j++) {
            if (M[j] < 0) continue;
            const T hn = (j + 1 < C) ? H[j + 1] : hr;
            if constexpr (DF) {
                const T hnl = (j + 1 < C) ? Hl[j + 1] : hrl;
                const fcoef f = UNIFORM ? fu : load_fcoef(block(j));
                df_e_update(E[j], El[j], hn - H[j], hnl - Hl[j], P[j], f);
            } else if constexpr (DFD) {
                const fcoef f = UNIFORM ? fu : load_fcoef(block(j));
                E[j] = fmaf(f.a, E[j], fmaf(f.bh, hn - H[j], -f.g * P[j]));
            } else {
                const T* cb = block(j);
                E[j] = cb[pre::FD_A] * E[j] +
                    cb[pre::FD_B] * (-cb[pre::FD_GAMMA] * P[j] + (hn - H[j]) * dxi);
            }
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
                    if (sd.type == 0) {
                        E[j] = (T) v;
                        if constexpr (DF) El[j] = (T) (v - (double) E[j]);
                    } else {
                        if constexpr (DF)
                            df_add(E[j], El[j], v);
                        else
                            E[j] += (T) v;
                    }
                }
            }
        }
        // ---- H: needs E (hi, lo) of the left neighbour
        if (lane == 31) {
            sh_b[warp] = E[C - 1];
            if constexpr (DF) sh_bl[warp] = El[C - 1];
        }
        __syncthreads();
        T el = __shfl_up_sync(0xffffffffu, E[C - 1], 1);
        T ell = DF ? __shfl_up_sync(0xffffffffu, El[C - 1], 1) : T(0);
        if (lane == 0) {
            el = (warp > 0) ? sh_b[warp - 1] : T(0);
            if constexpr (DF) ell = (warp > 0) ? sh_bl[warp - 1] : T(0);
        }
#pragma unroll
        for (int j = 0; j < C; j++) {
            const int64_t l = l0 + j;
            if (l >= 1 && l < nx) {
                const T ep = (j > 0) ? E[j - 1] : el;
                if constexpr (DF) {
                    const T epl = (j > 0) ? El[j - 1] : ell;
                    const fcoef f = UNIFORM ? fu : load_fcoef(block(j));
                    df_h_update(H[j], Hl[j], E[j] - ep, El[j] - epl, f);
                } else if constexpr (DFD) {
                    const fcoef f = UNIFORM ? fu : load_fcoef(block(j));
                    H[j] = fmaf(f.ch, E[j] - ep, H[j]);
                } else {
                    H[j] += block(j)[pre::FD_C] * (E[j] - ep);
                }
            } else if (l == 0) {
                H[j] = T(0);  // PMC (solver_cpu_fdtd.tpp:273)
                if constexpr (DF) Hl[j] = T(0);
            }
        }
        if (!UNIFORM && tl.wall) {
            // mirror walls (the thread holding point 0 or the point beyond
            // the right end): H = k_left E[0] before the left end,
            // -k_right E[nx - 1] beyond the right end (a point of zero
            // state, never updated or stored), read by the end points' E
            // updates in the next step. The flag lives in shared memory and
            // the coefficients are read here: values held in registers
            // across the time loop cost the 2-level kernel its register
            // budget (coefficients reloaded every step).
            const run_desc& rw = p.runs[td.run];
            const T k_left = (T) rw.k_left, k_right = (T) rw.k_right;
#pragma unroll
            for (int j = 0; j < C; j++) {
                const int64_t l = l0 + j;
                if (l == 0 && k_left != T(0)) {
                    H[j] = k_left * E[j];
                    if constexpr (DF) Hl[j] = k_left * El[j];
                } else if (l == nx && k_right != T(0)) {
                    H[j] = -k_right * ((j > 0) ? E[j - 1] : el);
                    if constexpr (DF) Hl[j] = -k_right * ((j > 0) ? El[j - 1] : ell);
                }
            }
        }
        // ---- density matrix and polarisation current at every point
        if constexpr (TCU) {
            // all threads take part in the CTA-wide products; threads
            // without a point pass zeros and keep their zero state
            if (qm_uniform) {
                const bool act = M[0] >= 0;
                const float e = act ? E[0] + El[0] : 0.0f;
                float pn = 0.0f;
                const tc::coef_small<D> cf{ sh_coef };
                if (!tc::cvr_update_df_tc<D>(*tcc, R[0], Rl[0], e, pn, cf)) return false;
                if (act) {
                    P[0] = pn;
                } else {
#pragma unroll
                    for (int v = 0; v < D; v++) R[0][v] = Rl[0][v] = T(0);
                }
            }
        } else if constexpr (D > 0) {
#pragma unroll
            for (int j = 0; j < C; j++) {
                if (M[j] < 0) continue;
                const T* cb = block(j);
                if (UNIFORM ? !qm_uniform : cb[pre::FD_HAS_QM] == T(0)) continue;
                const T e = DF ? E[j] + El[j] : E[j];
                if constexpr (ALGO == 1) {
                    if constexpr (REGCOEF) {
                        if constexpr (DFD)
                            cvr_update_df<D>(R[j], Rl[j], e, P[j], creg);
                        else
                            cvr_update<T, D>(R[j], e, P[j], creg);
                    } else if constexpr (TC) {
                        // mixed tile of the tensor-core kernel: in place
                        // through this thread's row of the idle A operand
                        cvr_coef<T, D> cf{ cb };
                        tc::cvr_update_df_row<D>(tcc->rows + threadIdx.x * D, R[j], Rl[j], e, P[j], cf);
                    } else if constexpr (PADC) {
                        const cvr_coef_pad<T, D> cf{ (uint32_t) __cvta_generic_to_shared(sh_coef), sh_coef };
                        if constexpr (DFD)
                            cvr_update_df<D>(R[j], Rl[j], e, P[j], cf);
                        else
                            cvr_update<T, D>(R[j], e, P[j], cf);
                    } else {
                        cvr_coef<T, D> cf{ cb };
                        if constexpr (DFD)
                            cvr_update_df<D>(R[j], Rl[j], e, P[j], cf);
                        else
                            cvr_update<T, D>(R[j], e, P[j], cf);
                    }
                } else if constexpr (DFD) {
                    cayley_update_df<LEV>(R[j], Rl[j], e, P[j], cb);
                } else {
                    cayley_update<T, LEV>(R[j], e, P[j], cb);
                }
            }
        }
        // ---- recording (solver_cpu_fdtd.tpp:288-325)
        if (p.record) {
            for (int r = 0; r < nrec; r++) {
                const rec_desc rc = tl.overflow ? p.recs[rd.rec_begin + r] : tl.rec[r];
                // every-step records (ratio 1) need no FP64 arithmetic
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
                    const T ev = DF ? E[j] + El[j] : E[j];
                    const T hv = DF ? H[j] + Hl[j] : H[j];
                    T v = T(0);
                    if constexpr (ALGO == 2) {
                        switch (rc.type) {
                        case 0: v = ev; break;
                        case 1: v = P[j]; break;
                        case 2: v = hv; break;
                        case 4: v = DFD ? (R[j][1] - R[j][0]) + (Rl[j][1] - Rl[j][0]) : R[j][1] - R[j][0]; break;
                        default: {
                            // populations (3) and coherence parts (REC_COH_*):
                            // an entry of the packed matrix (diagonal, then
                            // the upper triangle as (re, im) pairs); constant
                            // indices keep R in registers
                            const uint32_t a = min(rc.row_idx, rc.col_idx);
                            const uint32_t b = max(rc.row_idx, rc.col_idx);
                            uint32_t idx = rc.type == 3 ? (a == b ? a : 0xffffffffu)
                                                        : LEV + 2 * (b * (b - 1) / 2 + a) +
                                                            (rc.type == REC_COH_IM ? 1 : 0);
#pragma unroll
                            for (int q = 0; q < LEV * LEV; q++)
                                if (idx == (uint32_t) q) v = DFD ? R[j][q] + Rl[j][q] : R[j][q];
                            if (rc.type == REC_COH_IM && rc.row_idx > rc.col_idx) v = -v;
                            break;
                        }
                        }
                    } else {
                        constexpr int DDv = D > 0 ? D : 1;
                        T u[DDv];
#pragma unroll
                        for (int q = 0; q < DDv; q++) u[q] = DFD ? R[j][q] + Rl[j][q] : R[j][q];
                        // the padded shared copy lacks the record rows, the
                        // staged copy the coherence rows
                        const T* rb = (PADC || rc.type >= REC_COH_RE) ? p.mc + (uint64_t) M[j] * p.mstride
                                                                       : block(j);
                        v = cvr_record_value<T, D>(rc, ev, hv, P[j], u, rb, LEV);
                    }
                    p.scratch[rc.offset + row * rc.cols + (uint64_t) (l - rc.pos)] = v;
                    if (!isfinite(v)) atomicOr(p.status, STATUS_NONFINITE);
                }
            }
        }
    }
    if (!UNIFORM && tl.wall) {
        // the point beyond the right end goes back to zero state (a bulk
        // store rounded up to 16 bytes may write it into the run's padding)
#pragma unroll
        for (int j = 0; j < C; j++)
            if (l0 + j == nx) {
                H[j] = T(0);
                if constexpr (DF) Hl[j] = T(0);
            }
    }
    return true;
}

// Tensor memory columns, completion barrier and its phase of a CTA of the
// tensor-core kernels (allocated once per CTA by the kernel wrappers).
struct tc_res {
    uint32_t tmem, mbar;
    uint32_t* phase;  // shared: the barrier's phase between tiles
};

__device__ __forceinline__ tc_res tc_acquire(uint32_t* tmem_sh, uint64_t* mbar, uint32_t* phase_sh)
{
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t) __cvta_generic_to_shared(tmem_sh)),
                     "r"(tc::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t) __cvta_generic_to_shared(mbar))
                     : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *phase_sh = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    return tc_res{ *tmem_sh, (uint32_t) __cvta_generic_to_shared(mbar), phase_sh };
}

__device__ __forceinline__ void tc_release(const tc_res& r)
{
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(r.tmem), "r"(tc::TMEM_COLS)
                     : "memory");
    }
}

// One tile of one launch: the tile advances by nsub steps. TC: 4-6 levels
// in FP32 with the density products of uniform tiles on the tensor cores.
// `flip` swaps the input and output buffers (odd levels of the persistent
// kernel); CG loads the state through L2 only (the persistent kernel reads
// what other CTAs of the same launch wrote).
template<typename T, int ALGO, int LEV, int C, int NT, bool TC, bool BULK = false, bool CG = false>
__device__ __forceinline__ void step_body(const kparams<T>& p, uint32_t tile, uint32_t launch_idx, bool flip,
                                          const tc_res& res)
{
    constexpr bool DF = sizeof(T) == 4;
    constexpr int D = density_len<ALGO, LEV>::value;
    constexpr int DD = D > 0 ? D : 1;
    constexpr int NW = NT / 32;
    constexpr bool DFD = DF && ALGO != 0;  // FP32 density state as float pairs
    __shared__ T sh_a[NW], sh_al[NW], sh_b[NW], sh_bl[NW];
    __shared__ tile_lists tl;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sh_coef = reinterpret_cast<T*>(smem_raw);

    const tile_desc td = p.tiles[tile];
    const run_desc rd = p.runs[td.run];
    const int64_t l0 = (int64_t) td.out_start - (int64_t) p.halo + (int64_t) threadIdx.x * C;
    const int64_t g0 = (int64_t) rd.offset + l0;
    const int64_t nx = rd.n_x;
    const uint64_t step0 = *p.step_base + (uint64_t) launch_idx * p.depth;
    const T* const Ein = flip ? p.Eout : p.Ein;
    const T* const Hin = flip ? p.Hout : p.Hin;
    const T* const Pin = flip ? p.Pout : p.Pin;
    const T* const Din = flip ? p.Dout : p.Din;
    const T* const Elin = flip ? p.Elout : p.Elin;
    const T* const Hlin = flip ? p.Hlout : p.Hlin;
    T* const Eout = flip ? const_cast<T*>(p.Ein) : p.Eout;
    T* const Hout = flip ? const_cast<T*>(p.Hin) : p.Hout;
    T* const Pout = flip ? const_cast<T*>(p.Pin) : p.Pout;
    T* const Dout = flip ? const_cast<T*>(p.Din) : p.Dout;
    T* const Elout = flip ? const_cast<T*>(p.Elin) : p.Elout;
    T* const Hlout = flip ? const_cast<T*>(p.Hlin) : p.Hlout;
    int nsteps = 0;
    if (step0 < rd.n_t) nsteps = (int) min((uint64_t) p.nsub, (uint64_t) rd.n_t - step0);

    // sources inside the tile's window (halo included: the halo points
    // must see them too) and records inside its output range
    if (threadIdx.x == 0) {
        const int64_t w0 = (int64_t) td.out_start - (int64_t) p.halo;
        const int64_t w1 = w0 + (int64_t) NT * C;
        int ns = 0, nr = 0, of = 0;
        for (uint32_t s = rd.src_begin; s < rd.src_end; s++) {
            const src_desc sd = p.srcs[s];
            if ((int64_t) sd.x_idx < w0 || (int64_t) sd.x_idx >= w1) continue;
            if (ns < TILE_MAX_SRC)
                tl.src[ns++] = sd;
            else
                of = 1;
        }
        for (uint32_t r = rd.rec_begin; r < rd.rec_end; r++) {
            const rec_desc rc = p.recs[r];
            const int64_t lo = max((int64_t) rc.pos, (int64_t) td.out_start);
            const int64_t hi = min((int64_t) rc.pos + rc.cols, (int64_t) td.out_start + td.out_len);
            if (lo >= hi) continue;
            if (nr < TILE_MAX_REC)
                tl.rec[nr++] = rc;
            else
                of = 1;
        }
        tl.nsrc = ns;
        tl.nrec = nr;
        tl.overflow = of;
        // a mirror wall inside the window: point 0 or the point beyond the
        // right end (index n_x)
        tl.wall = (rd.k_left != 0.0 && w0 <= 0 && 0 < w1) ||
            (rd.k_right != 0.0 && w0 <= (int64_t) rd.n_x && (int64_t) rd.n_x < w1);
    }

    T E[C], El[C], H[C], Hl[C], P[C];
    T R[C][DD];
    T Rl[C][DD];  // FP32 coherence vector: low words
    int32_t M[C];
    // BULK: the tile's state planes are staged in shared memory with bulk
    // asynchronous copies (TMA); otherwise they load straight into registers
    static_assert(!BULK || bulk::enabled<T, ALGO, LEV, TC>(), "bulk staging: 2-level FP32 only");
    __shared__ __align__(8) uint64_t bulk_mbar;
    uint32_t bulk_s = 0;
    float* bulk_g = nullptr;
    if constexpr (BULK) {
        const uint32_t sraw = (uint32_t) __cvta_generic_to_shared(smem_raw);
        bulk_s = (sraw + (uint32_t) (p.mstage * sizeof(T)) + 127u) & ~127u;
        bulk_g = reinterpret_cast<float*>(smem_raw + (bulk_s - sraw));
        const uint64_t gt = (uint64_t) ((int64_t) rd.offset + (int64_t) td.out_start - (int64_t) p.halo);
        const bool ok = bulk::load<D, NT * C>(p, gt, (uint32_t) __cvta_generic_to_shared(&bulk_mbar), bulk_s);
        if (!ok) {
            if (threadIdx.x == 0) atomicOr(p.status, STATUS_TC_WAIT);
            return;
        }
        const float* mine = bulk_g + threadIdx.x * C;
        bulk::take<C>(E, mine, 0, NT * C);
        bulk::take<C>(H, mine, 1, NT * C);
        bulk::take<C>(P, mine, 2, NT * C);
        bulk::take<C>(El, mine, 3, NT * C);
        bulk::take<C>(Hl, mine, 4, NT * C);
#pragma unroll
        for (int v = 0; v < D; v++) {
            T tmp[C];
            bulk::take<C>(tmp, mine, 5 + v, NT * C);
#pragma unroll
            for (int j = 0; j < C; j++) R[j][v] = tmp[j];
            bulk::take<C>(tmp, mine, 5 + D + v, NT * C);
#pragma unroll
            for (int j = 0; j < C; j++) Rl[j][v] = tmp[j];
        }
    } else {
        load_cells<T, C, CG>(E, Ein, g0);
        load_cells<T, C, CG>(H, Hin, g0);
        load_cells<T, C, CG>(P, Pin, g0);
        if constexpr (DF) {
            load_cells<T, C, CG>(El, Elin, g0);
            load_cells<T, C, CG>(Hl, Hlin, g0);
        }
        if constexpr (D > 0) {
#pragma unroll
            for (int v = 0; v < D; v++) {
                T tmp[C];
                load_cells<T, C, CG>(tmp, Din + (uint64_t) v * p.plane, g0);
#pragma unroll
                for (int j = 0; j < C; j++) R[j][v] = tmp[j];
                if constexpr (DFD) {
                    load_cells<T, C, CG>(tmp, Din + (uint64_t) (D + v) * p.plane, g0);
#pragma unroll
                    for (int j = 0; j < C; j++) Rl[j][v] = tmp[j];
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < C; j++) {
        if constexpr (!DFD)
#pragma unroll
            for (int v = 0; v < DD; v++) Rl[j][v] = T(0);
        const int64_t l = l0 + j;
        const bool valid = (l >= 0) && (l < nx);
        M[j] = valid ? __ldg(p.mat + g0 + j) : -1;
        if (!valid) {
            E[j] = H[j] = P[j] = T(0);
            El[j] = Hl[j] = T(0);
#pragma unroll
            for (int v = 0; v < DD; v++) R[j][v] = Rl[j][v] = T(0);
        }
        if constexpr (!DF) El[j] = Hl[j] = T(0);
    }
    tc::ctx tcc{};
    const bool uniform = td.uniform_mat >= 0;
    if (uniform) {
        const T* src = p.mc + (uint64_t) td.uniform_mat * p.mstride;
        if constexpr (TC) {
            using Ls = tc::coef_small<D>;
            for (int i = threadIdx.x; i < Ls::len; i += NT) sh_coef[i] = src[Ls::source(i)];
        } else if constexpr (ALGO == 1 && D >= 15) {
            using Lp = cvr_pad<T, D>;
            for (int i = threadIdx.x; i < Lp::len; i += NT) {
                const int q = Lp::source(i);
                sh_coef[i] = q >= 0 ? src[q] : T(0);
            }
        } else {
            for (int i = threadIdx.x; i < (int) p.mstage; i += NT) sh_coef[i] = src[i];
        }
    }
    __syncthreads();

    if constexpr (TC) {
        tc::fence_after();
        const uint32_t sbase = (uint32_t) __cvta_generic_to_shared(smem_raw);
        const uint32_t ops = (sbase + (uint32_t) (tc::coef_small<D>::len * sizeof(T)) + 127u) & ~127u;
        tcc.rows = reinterpret_cast<float*>(smem_raw + (ops - sbase));
        using TS = tc::shape<D>;
        tcc.a_hi = ops;
        tcc.a_lo = ops + TS::A_BYTES;
        tcc.b_hi = ops + 2u * TS::A_BYTES;
        tcc.b_lo = tcc.b_hi + TS::B_BYTES;
        tcc.b_dl = tcc.b_lo + TS::B_BYTES;
        tcc.tmem = res.tmem;
        tcc.mbar = res.mbar;
        tcc.phase = *res.phase;
        tcc.wait_limit = p.wait_limit ? p.wait_limit : tc::WAIT_LIMIT;
        if (uniform) tc::stage_b<D>(tcc, p.mc + (uint64_t) td.uniform_mat * p.mstride);
    }

    if (uniform) {
        if constexpr (pair_path<T, ALGO, LEV, C, TC>()) {
            // two points per instruction (pair_steps.cuh)
            if (cvr2_sparse(sh_coef))
                tile_steps_pair<C, NT, true>(p, td, rd, l0, nsteps, step0, E, H, P, R, Rl, M, sh_coef, tl, sh_a, sh_b);
            else
                tile_steps_pair<C, NT, false>(p, td, rd, l0, nsteps, step0, E, H, P, R, Rl, M, sh_coef, tl, sh_a,
                                              sh_b);
        } else {
            const bool ok = tile_steps<T, ALGO, LEV, C, NT, true, TC>(p, td, rd, l0, nsteps, step0, E, El, H, Hl,
                                                                      P, R, Rl, M, sh_coef, tl, sh_a, sh_al,
                                                                      sh_b, sh_bl, &tcc);
            if (!ok && threadIdx.x == 0) atomicOr(p.status, STATUS_TC_WAIT);
        }
    } else {
        tile_steps<T, ALGO, LEV, C, NT, false>(p, td, rd, l0, nsteps, step0, E, El, H, Hl, P, R, Rl, M,
                                               sh_coef, tl, sh_a, sh_al, sh_b, sh_bl);
    }
    if constexpr (TC) {
        // every thread holds the same phase; the next tile of a persistent
        // CTA continues from it (the barrier before its first product
        // orders this write)
        if (threadIdx.x == 0) *res.phase = tcc.phase;
    }

    // Cayley, FP32: renormalise the trace to that of the initial density
    // matrix, in FP64, once per launch (the exact propagators preserve it:
    // the scattering matrix has zero column sums and U2 is unitary; this
    // removes FP32 round-off drift). The pairs take the scaling as an
    // increment, (s - 1) rho, accumulated error-free.
    if constexpr (ALGO == 2 && DF) {
        const pre::cay_layout L = pre::make_cay_layout(LEV);
#pragma unroll
        for (int j = 0; j < C; j++) {
            if (M[j] < 0 || nsteps == 0) continue;
            const T* cb = uniform ? sh_coef : p.mc + (uint64_t) M[j] * p.mstride;
            if (cb[pre::FD_HAS_QM] == T(0)) continue;
            double tr = 0.0, target = 0.0;
#pragma unroll
            for (int i = 0; i < LEV; i++) {
                tr += (double) R[j][i] + (double) Rl[j][i];
                target += (double) cb[L.rho0 + i];
            }
            if (tr != 0.0 && fabs(tr / target - 1.0) < 1e-3) {
                const float ds = (float) (target / tr - 1.0);
#pragma unroll
                for (int v = 0; v < DD; v++) {
                    df_acc(R[j][v], Rl[j][v], ds * R[j][v], ds * Rl[j][v]);
                    df_renorm(R[j][v], Rl[j][v]);
                }
            }
        }
    }

    if constexpr (BULK) {
        // every thread puts its cells back into the staged planes; one thread
        // writes the tile's output range to global memory with bulk copies
        float* mine = bulk_g + threadIdx.x * C;
        bulk::give<C>(E, mine, 0, NT * C);
        bulk::give<C>(H, mine, 1, NT * C);
        bulk::give<C>(P, mine, 2, NT * C);
        bulk::give<C>(El, mine, 3, NT * C);
        bulk::give<C>(Hl, mine, 4, NT * C);
#pragma unroll
        for (int v = 0; v < D; v++) {
            T tmp[C];
#pragma unroll
            for (int j = 0; j < C; j++) tmp[j] = R[j][v];
            bulk::give<C>(tmp, mine, 5 + v, NT * C);
#pragma unroll
            for (int j = 0; j < C; j++) tmp[j] = Rl[j][v];
            bulk::give<C>(tmp, mine, 5 + D + v, NT * C);
        }
        bulk::store<D, NT * C>(p, (uint64_t) rd.offset + (uint64_t) td.out_start, (uint32_t) td.out_len,
                               bulk_s + (uint32_t) (p.halo * sizeof(float)));
        return;
    }
    const int64_t lo = td.out_start, hi = (int64_t) td.out_start + td.out_len;
    store_cells<T, C>(E, Eout, g0, l0, lo, hi);
    store_cells<T, C>(H, Hout, g0, l0, lo, hi);
    store_cells<T, C>(P, Pout, g0, l0, lo, hi);
    if constexpr (DF) {
        store_cells<T, C>(El, Elout, g0, l0, lo, hi);
        store_cells<T, C>(Hl, Hlout, g0, l0, lo, hi);
    }
    if constexpr (D > 0) {
#pragma unroll
        for (int v = 0; v < D; v++) {
            T tmp[C];
#pragma unroll
            for (int j = 0; j < C; j++) tmp[j] = R[j][v];
            store_cells<T, C>(tmp, Dout + (uint64_t) v * p.plane, g0, l0, lo, hi);
            if constexpr (DFD) {
#pragma unroll
                for (int j = 0; j < C; j++) tmp[j] = Rl[j][v];
                store_cells<T, C>(tmp, Dout + (uint64_t) (D + v) * p.plane, g0, l0, lo, hi);
            }
        }
    }
}

// The time-step kernels. The CUDA-core kernels leave the register budget to
// the compiler (a minimum-blocks hint would raise the 2-level kernels to
// more registers and one CTA per SM); the tensor-core kernels ask for 3
// CTAs per SM (4 for 4 levels), which needs the in-place update's budget.
template<typename T, int ALGO, int LEV, int C, int NT>
__global__ void __launch_bounds__(NT) step_kernel(const kparams<T> p)
{
    step_body<T, ALGO, LEV, C, NT, false>(p, blockIdx.x, p.launch_idx, false, tc_res{});
}

template<int LEV>
__global__ void __launch_bounds__(tc::M, LEV <= 4 ? 4 : 3) step_kernel_tc(const kparams<float> p)
{
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_sh, phase_sh;
    const tc_res r = tc_acquire(&tmem_sh, &mbar, &phase_sh);
    step_body<float, 1, LEV, 1, tc::M, true>(p, blockIdx.x, p.launch_idx, false, r);
    tc_release(r);
}

// 2-level FP32 kernels with bulk-copy (TMA) staging of the tile state; not
// the default (measured slower on this issue-bound kernel), selected by
// MBG_TILE_STAGING=bulk
template<int C, int NT>
__global__ void __launch_bounds__(NT) step_kernel_bulk(const kparams<float> p)
{
    step_body<float, 1, 2, C, NT, false, true>(p, blockIdx.x, p.launch_idx, false, tc_res{});
}

// ------------------------------------------------------- persistent kernel
//
// One launch runs q.levels launches' worth of tiles ("levels" of nsub
// steps). The CTAs take work items w = level * n_tiles + tile from a
// global counter, in order, until none is left. A tile of
// level k reads what its own tile and its two neighbours (the only tiles
// whose outputs its window overlaps: a halo is at most half an output
// range) wrote at level k - 1, and overwrites a buffer those three read at
// level k - 1: it waits until all three have finished level k - 1
// (per-tile progress counters, absolute over the launches so that nothing
// is reset between launches). Items are taken in order, so every item
// waited for was taken earlier by a running CTA (a CTA takes items only
// while it runs) and finishes: no deadlock, whether or not every CTA of the
// grid is resident at once. Waits are bounded; a time-out sets STATUS_PERSIST_WAIT.
// Results equal the launch-per-level kernels' bit for bit (same tiles,
// same arithmetic); what goes away is the wave quantisation and the gaps
// between launches (long single runs have only 1-3 waves of tiles).

constexpr uint32_t PERSIST_WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* a)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
    return v;
}

// until the three progress counters reach `need` (polled together, at most
// `limit` times), then an acquire fence; false when the wait ran out
__device__ __forceinline__ bool wait_progress(const uint32_t* a, const uint32_t* b, const uint32_t* c,
                                              uint32_t need, uint32_t limit)
{
    for (uint32_t it = 0; it < limit; it++) {
        const uint32_t va = ld_relaxed(a), vb = ld_relaxed(b), vc = ld_relaxed(c);
        if ((int32_t) (va - need) >= 0 && (int32_t) (vb - need) >= 0 && (int32_t) (vc - need) >= 0) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            return true;
        }
        __nanosleep(32);
    }
    return false;
}

template<typename T, int ALGO, int LEV, int C, int NT, bool TC>
__device__ __forceinline__ void persist_loop(const kparams<T>& p, const persist_params& q, const tc_res& r)
{
    __shared__ uint32_t w_sh;
    const uint32_t total = q.levels * q.n_tiles;
    if (threadIdx.x == 0) w_sh = atomicAdd(q.work, 1u);
    __syncthreads();
    for (;;) {
        const uint32_t w = w_sh;
        if (w >= total) break;  // the same in every thread
        const uint32_t k = w / q.n_tiles, i = w - k * q.n_tiles;
        if (threadIdx.x == 0) {
            const int2 nb = q.nb[i];
            // q.stall (tests only) asks for progress no tile reaches
            if (!wait_progress(q.prog + i, q.prog + nb.x, q.prog + nb.y, q.base + k + q.stall,
                               q.wait_limit ? q.wait_limit : PERSIST_WAIT_LIMIT))
                atomicOr(p.status, STATUS_PERSIST_WAIT);
        }
        __syncthreads();
        step_body<T, ALGO, LEV, C, NT, TC, false, true>(p, i, k, (k & 1u) != 0, r);
        // the CTA's stores, then (one thread) a release fence and the
        // progress mark; the next item is fetched meanwhile
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(q.prog + i), "r"(q.base + k + 1)
                         : "memory");
            w_sh = atomicAdd(q.work, 1u);
        }
        __syncthreads();
    }
}

template<typename T, int ALGO, int LEV, int C, int NT>
__global__ void __launch_bounds__(NT) step_kernel_persist(const kparams<T> p, const persist_params q)
{
    persist_loop<T, ALGO, LEV, C, NT, false>(p, q, tc_res{});
}

template<int LEV>
__global__ void __launch_bounds__(tc::M, LEV <= 4 ? 4 : 3)
    step_kernel_persist_tc(const kparams<float> p, const persist_params q)
{
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_sh, phase_sh;
    const tc_res r = tc_acquire(&tmem_sh, &mbar, &phase_sh);
    persist_loop<float, 1, LEV, 1, tc::M, true>(p, q, r);
    tc_release(r);
}

}  // namespace mbg
