// FP64 precompute of the per-material constants the time-step kernels use.
//
// One code path for host and device (__host__ __device__): the solvers run
// it on the GPU, one thread per material; tests without a GPU run the host
// instantiation through mbg_material_constants().
//
// Coherence-vector / Rodrigues form (algo_lindblad_cvr_rodr.hpp:143-229,
// coherence_vector_representation.hpp:52-213). The reference advances the
// coherence vector d by
//     d1 = A1 (d + d_in) - d_in,  d2 = A2(e) d1,  d = A1 (d2 + d_in) - d_in
// with A1 = exp(M dt/2) and A2(e) = exp(e dt U), U skew-symmetric, A2 built
// from the real-Schur planes of U. Here the state is the same vector in the
// basis Q of those planes, u = Q^T d. With F = A1 - I and the small
// constant kh = Q^T F d_in (A1 d + F d_in is the reference's first half
// step), one step is
//     w = u + (Bh u + kh);  w <- R(e) w;  u = w + (Bh w + kh)
// with Bh = Q^T F Q and R(e) block-diagonal with a 2x2 rotation by
// theta_k e dt per plane and the identity on the null space of U: V/2 plane
// rotations per point instead of forming A2. The second half step of one
// step and the first of the next merge into one full step, so the kernels
// keep v = u + (Bh u + kh) and do one product per step (cvr_layout):
//     v <- R(e) v;  v = v + (Bd v + k),  Bd = Q^T (exp(M dt) - I) Q.
// The polarisation current p_t = M_CP v_dip^T (M d + d_eq) is g^T u + p0
// with g = M_CP Q^T M^T v_dip and p0 = M_CP v_dip^T d_eq, composed with
// u = A1^-1 (v - kh) into a row on v. Every stage adds a small correction
// to a vector of norm about 1; Bd comes from exp(X) - I computed directly.
// The FP32 kernels keep v as a float pair (hi + lo), add the corrections
// with TwoSum and add Bdl = Bd - fl32(Bd) into the low word: otherwise the
// FP32 rounding of Bd acts as a systematic shift of the transition
// frequency.
//
// Planes of U: U is real skew-symmetric, so i U is complex Hermitian with
// eigenvalues +-theta_k; an eigenvector a + i b for +theta gives the
// orthonormal pair q1 = sqrt2 a, q2 = sqrt2 b with U q1 = theta q2,
// U q2 = -theta q1. Eigen-decomposition by the cyclic complex Jacobi method
// (Golub & Van Loan, Matrix Computations, 4th ed., sec. 8.5, with the
// complex phase rotation for Hermitian matrices); the null space is
// completed by Gram-Schmidt against the unit vectors.
//
// Matrix exponential: scaling and squaring with a truncated Taylor series
// (Moler & Van Loan, "Nineteen dubious ways to compute the exponential of
// a matrix", method 3 with scaling and squaring), evaluated as exp(X) - I
// and squared with F <- F (F + 2I) so that exp(X) - I keeps its relative
// accuracy for small X.
//
// Regular / Cayley form (algo_lindblad_reg_cayley.hpp:123-203): the kernel
// uses kappa H0 and kappa mu (kappa = dt/(2 hbar)), D1 - I with
// D1 = exp(S dt/2), D2 - 1 = expm1(gamma dt/2), H0/hbar and n mu.
#pragma once

#include "common.cuh"

namespace mbg {
namespace pre {

// One material, flattened (FP64, SI units). Operators are full N x N.
struct mat_in {
    int32_t N;           // 0: no quantum-mechanical description
    int32_t relax_kind;  // MBG_RELAX_*
    int32_t rho_levels;
    int32_t rho_num_off;  // off-diagonal entries of the initial rho (<= 15 kept)
    double eps_r, mu_r, overlap, losses;
    double carrier_density;
    double dt, dx;
    double h_re[36], h_im[36];
    double mu_re[36], mu_im[36];
    double S[36];        // scattering, row-major
    double deph[15];     // packed upper triangle, column-major order
    double rho_diag[6];
    double rho_off_re[15], rho_off_im[15];
};

struct cd {
    double re, im;
};
MBG_HD cd cmake(double r, double i) { return cd{ r, i }; }
MBG_HD cd cadd(cd a, cd b) { return cd{ a.re + b.re, a.im + b.im }; }
MBG_HD cd csub(cd a, cd b) { return cd{ a.re - b.re, a.im - b.im }; }
MBG_HD cd cmul(cd a, cd b)
{
    return cd{ a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re };
}
MBG_HD cd cconj(cd a) { return cd{ a.re, -a.im }; }

// ------------------------------------------------------------- layouts

// Leading FDTD part of every material block (both algorithms):
//   0 a, 1 b, 2 c, 3 Gamma       (common_fdtd.hpp:131-190)
//   4 has_qm, 5 p0 (CVR), 6 nplanes (CVR), 7 unused
//   8 b/dx, 9 b/dx - fl32(b/dx), 10 c - fl32(c), 11 b Gamma
// Entries 8-11 serve the FP32 kernels, which keep E and H as unevaluated
// sums of two floats and need the coefficients to the same accuracy.
enum : int {
    FD_A = 0,
    FD_B = 1,
    FD_C = 2,
    FD_GAMMA = 3,
    FD_HAS_QM = 4,
    FD_BDX = 8,
    FD_BDX_LO = 9,
    FD_C_LO = 10,
    FD_G = 11,
    FDTD_END = 12
};

// Constant block of one material for the coherence-vector kernels.
//
// The reference's step (rodr.hpp:234-268) is, in the plane basis u = Q^T d,
//   u <- A u + kh;  u <- R(e) u;  u <- A u + kh
// with A = exp(M dt/2) and kh = (A - I) d_in. Two consecutive steps meet
// in A (A u + kh) + kh = A^2 u + (A^2 - I) d_in: the kernels therefore keep
// the state one half step ahead, v = A u + kh, and advance it by
//   v <- R(e) v;  v <- v + (Bd v + k)
// with Bd = A^2 - I = Q^T (exp(M dt) - I) Q and k = Q^T (exp(M dt) - I) d_in:
// one matrix product per step instead of two. u = A^-1 (v - kh) is never
// formed: P = p0 + g . v and the records' rows (inv, pop) are composed with
// A^-1 and kh here, and the initial state z0 is v0 = A u0 + kh. Bh and kh
// (the half step) are kept after Q for inspection.
struct cvr_layout {
    int N, V, KP;
    int a, b, cH, gam, has_qm, p0, nplanes;
    int Bd, Bdl, k, g, thdt, z0, inv, inv_c, pop, pop_c;
    int Q;       // the plane basis (inspection only; kernels stop before it)
    int Bh, kh;  // the half step (inspection only)
    // coherence records: rho[j][k] (j < k, pair q = k(k-1)/2 + j) is
    // coh[(2q) V ..] . v + coh_c[2q] + i (coh[(2q+1) V ..] . v + coh_c[2q+1])
    int coh, coh_c;
    int stage;   // leading part a kernel stages in shared memory
    int stride;
};

MBG_HD cvr_layout make_cvr_layout(int N)
{
    cvr_layout L;
    L.N = N;
    L.V = (N > 0) ? N * N - 1 : 0;
    L.KP = L.V / 2;
    L.a = 0;
    L.b = 1;
    L.cH = 2;
    L.gam = 3;
    L.has_qm = 4;
    L.p0 = 5;
    L.nplanes = 6;
    int o = FDTD_END;
    L.Bd = o;
    o += L.V * L.V;
    L.Bdl = o;  // Bd - fl32(Bd): the FP32 kernels add it to the low word
    o += L.V * L.V;
    L.k = o;
    o += L.V;
    L.g = o;
    o += L.V;
    L.thdt = o;
    o += (L.KP > 0 ? L.KP : 1);
    L.z0 = o;
    o += L.V;
    L.inv = o;
    o += L.V;
    L.inv_c = o;
    o += 1;
    L.pop = o;
    o += N * L.V;
    L.pop_c = o;
    o += N;
    L.stage = (o + 3) & ~3;
    L.Q = L.stage;
    o = L.Q + L.V * L.V;
    L.Bh = o;
    o += L.V * L.V;
    L.kh = o;
    o += L.V;
    const int P = N * (N - 1) / 2;
    L.coh = o;
    o += 2 * P * L.V;
    L.coh_c = o;
    o += 2 * P;
    L.stride = (o + 3) & ~3;
    return L;
}

// Constant block of one material for the Cayley kernels. Hermitian
// operators are packed as N real diagonal entries followed by the upper
// triangle in column-major order as (re, im) pairs: N^2 reals.
//
// The FP64 kernels follow the reference's step (reg_cayley.hpp:228-257)
// with the entries up to `stage64`. The FP32 kernels split the step into
// its field-free part and a field-dependent correction. With
// A(e) = I + i kappa (H0 - e mu), U2(e) = A(e)^-1 (I - i kappa (H0 - e mu))
// = 2 A(e)^-1 - I and D the dissipation half step,
//   rho <- D Ad(U2(e)) D rho = T0 rho + D(E(D rho)),
//   T0 = D Ad(U0) D (U0 = U2(0)),
//   E(s) = Ad(U2) s - Ad(U0) s = Z U2^H + U0 Z^H,  Z = dU s,
//   dU = U2(e) - U0 = 2 i e A(e)^-1 W,  W = kappa mu A(0)^-1.
// T0 - I (B0, a real N^2 x N^2 matrix on packed coordinates) is computed
// here in FP64 and stored as a float pair (B0 and B0l = B0 - fl32(B0)), so
// the free evolution that dominates every step carries no FP32 rounding
// (in FP32 it shifts the transition frequencies by ~1e-7 relative, which
// over 1e5 steps is a phase error far above 1e-5); dU is proportional to e
// and only needs FP32's relative accuracy. Full complex matrices are
// stored row-major as N^2 real parts then N^2 imaginary parts; B0 rows are
// padded to a multiple of 4 entries.
struct cay_layout {
    int N, P;
    int a, b, cH, gam, has_qm;
    int kH0, kMu, W0, Mn, dD1, d1, dD2, d2, rho0, gP;
    int stage64;  // leading part the FP64 kernels use and stage
    int U0, Wk, NP, B0, B0l;
    int blockB0;  // 1: H0 is diagonal and B0 block-diagonal (see cay_free_step)
    int stride;
};

MBG_HD cay_layout make_cay_layout(int N)
{
    cay_layout L;
    L.N = N;
    L.P = N * (N - 1) / 2;
    L.a = 0;
    L.b = 1;
    L.cH = 2;
    L.gam = 3;
    L.has_qm = 4;
    int o = FDTD_END;
    L.kH0 = o;
    o += N * N;
    L.kMu = o;
    o += N * N;
    L.W0 = o;
    o += N * N;
    L.Mn = o;
    o += N * N;
    L.dD1 = o;
    o += N * N;
    L.d1 = o;
    o += N * N;
    L.dD2 = o;
    o += (L.P > 0 ? L.P : 1);
    L.d2 = o;
    o += (L.P > 0 ? L.P : 1);
    L.rho0 = o;
    o += N * N;
    L.gP = o;  // P = gP . (packed density matrix)
    o += N * N;
    o = (o + 3) & ~3;
    L.stage64 = o;
    L.U0 = o;
    o += 2 * N * N;
    L.Wk = o;
    o += 2 * N * N;
    o = (o + 3) & ~3;
    L.NP = (N * N + 3) & ~3;
    L.B0 = o;
    o += N * N * L.NP;
    L.B0l = o;
    o += N * N * L.NP;
    L.blockB0 = o;
    o += 1;
    L.stride = (o + 3) & ~3;
    return L;
}

// Packed index of the upper off-diagonal entry (j, k), j < k, in
// column-major order: (0,1), (0,2), (1,2), (0,3), ...
MBG_HD int upper_index(int j, int k) { return k * (k - 1) / 2 + j; }

// --------------------------------------------------------- small linalg

// C = A * B, n x n row-major
MBG_HD void mat_mul(const double* A, const double* B, double* C, int n)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += A[i * n + k] * B[k * n + j];
            C[i * n + j] = s;
        }
}

MBG_HD double norm1(const double* A, int n)
{
    double m = 0.0;
    for (int j = 0; j < n; j++) {
        double s = 0.0;
        for (int i = 0; i < n; i++) s += fabs(A[i * n + j]);
        m = s > m ? s : m;
    }
    return m;
}

// F = exp(X) - I by scaling and squaring of a truncated Taylor series.
// ws: 3 n^2 doubles.
MBG_HD void expm_minus_identity(const double* X, double* F, int n, double* ws)
{
    double* Y = ws;
    double* T = ws + n * n;
    double* W = ws + 2 * n * n;
    double nrm = norm1(X, n);
    int s = 0;
    while (nrm > 0.25 && s < 200) {
        nrm *= 0.5;
        s++;
    }
    double scale = ldexp(1.0, -s);
    for (int i = 0; i < n * n; i++) Y[i] = X[i] * scale;
    // degree: smallest m with nrm^(m+1)/(m+1)! below 2^-60
    int m = 1;
    double term = nrm;
    while (m < 24) {
        term *= nrm / (m + 1);
        if (term < 8.7e-19) break;
        m++;
    }
    // F = Y (I + Y/2 (I + Y/3 (... (I + Y/m))))  (Horner form of e^Y - I)
    for (int i = 0; i < n * n; i++) T[i] = 0.0;
    for (int k = m; k >= 1; k--) {
        // T <- Y (I + T) / k   (T holds the bracket without its identity)
        for (int i = 0; i < n; i++) T[i * n + i] += 1.0;
        mat_mul(Y, T, W, n);
        for (int i = 0; i < n * n; i++) T[i] = W[i] / k;
    }
    for (int i = 0; i < n * n; i++) F[i] = T[i];
    // squaring: e^{2Y} - I = F (F + 2 I)
    for (int q = 0; q < s; q++) {
        for (int i = 0; i < n * n; i++) T[i] = F[i];
        for (int i = 0; i < n; i++) T[i * n + i] += 2.0;
        mat_mul(F, T, W, n);
        for (int i = 0; i < n * n; i++) F[i] = W[i];
    }
}

// Solve A x = b by Gaussian elimination with partial pivoting (A, b are
// overwritten). Returns 0, or 1 if a pivot is exactly zero.
MBG_HD int solve_partial_pivot(double* A, double* b, double* x, int n)
{
    int singular = 0;
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int i = k + 1; i < n; i++)
            if (fabs(A[i * n + k]) > fabs(A[p * n + k])) p = i;
        if (p != k) {
            for (int j = 0; j < n; j++) {
                double t = A[k * n + j];
                A[k * n + j] = A[p * n + j];
                A[p * n + j] = t;
            }
            double t = b[k];
            b[k] = b[p];
            b[p] = t;
        }
        double piv = A[k * n + k];
        if (piv == 0.0) {
            singular = 1;
            continue;
        }
        for (int i = k + 1; i < n; i++) {
            double f = A[i * n + k] / piv;
            for (int j = k; j < n; j++) A[i * n + j] -= f * A[k * n + j];
            b[i] -= f * b[k];
        }
    }
    for (int k = n - 1; k >= 0; k--) {
        double piv = A[k * n + k];
        if (piv == 0.0) {
            x[k] = 0.0;
            continue;
        }
        double s = b[k];
        for (int j = k + 1; j < n; j++) s -= A[k * n + j] * x[j];
        x[k] = s / piv;
    }
    return singular;
}

// Cyclic Jacobi eigen-decomposition of a complex Hermitian n x n matrix
// (re/im row-major, overwritten; the diagonal ends as the eigenvalues).
// Eigenvectors are the columns of (vre, vim).
MBG_HD void jacobi_hermitian(
    double* are,
    double* aim,
    double* vre,
    double* vim,
    int n)
{
    for (int i = 0; i < n * n; i++) {
        vre[i] = (i % (n + 1) == 0) ? 1.0 : 0.0;
        vim[i] = 0.0;
    }
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double m2 = are[i * n + j] * are[i * n + j] +
                    aim[i * n + j] * aim[i * n + j];
                tot += m2;
                if (i != j) off += m2;
            }
        if (off <= 1e-32 * tot) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double zr = are[p * n + q], zi = aim[p * n + q];
                double r = sqrt(zr * zr + zi * zi);
                if (r == 0.0) continue;
                double ephr = zr / r, ephi = zi / r;  // e^{i phi}
                double app = are[p * n + p], aqq = are[q * n + q];
                double tau = (aqq - app) / (2.0 * r);
                double t = (tau >= 0 ? 1.0 : -1.0) /
                    (fabs(tau) + sqrt(1.0 + tau * tau));
                double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
                // J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] on (p, q)
                // columns: X <- X J
                for (int k = 0; k < n; k++) {
                    double xpr = are[k * n + p], xpi = aim[k * n + p];
                    double xqr = are[k * n + q], xqi = aim[k * n + q];
                    // e^{-i phi} x_q
                    double yr = ephr * xqr + ephi * xqi;
                    double yi = ephr * xqi - ephi * xqr;
                    are[k * n + p] = c * xpr - s * yr;
                    aim[k * n + p] = c * xpi - s * yi;
                    are[k * n + q] = s * xpr + c * yr;
                    aim[k * n + q] = s * xpi + c * yi;
                }
                // rows: X <- J^H X
                for (int k = 0; k < n; k++) {
                    double xpr = are[p * n + k], xpi = aim[p * n + k];
                    double xqr = are[q * n + k], xqi = aim[q * n + k];
                    // e^{+i phi} x_q
                    double yr = ephr * xqr - ephi * xqi;
                    double yi = ephr * xqi + ephi * xqr;
                    are[p * n + k] = c * xpr - s * yr;
                    aim[p * n + k] = c * xpi - s * yi;
                    are[q * n + k] = s * xpr + c * yr;
                    aim[q * n + k] = s * xpi + c * yi;
                }
                are[p * n + q] = aim[p * n + q] = 0.0;
                are[q * n + p] = aim[q * n + p] = 0.0;
                aim[p * n + p] = aim[q * n + q] = 0.0;
                for (int k = 0; k < n; k++) {
                    double xpr = vre[k * n + p], xpi = vim[k * n + p];
                    double xqr = vre[k * n + q], xqi = vim[k * n + q];
                    double yr = ephr * xqr + ephi * xqi;
                    double yi = ephr * xqi - ephi * xqr;
                    vre[k * n + p] = c * xpr - s * yr;
                    vim[k * n + p] = c * xpi - s * yi;
                    vre[k * n + q] = s * xpr + c * yr;
                    vim[k * n + q] = s * xpi + c * yi;
                }
            }
    }
}

// --------------------------------------------------- SU(N) generators

// Sparse entries of generator i of su(N) in the reference's order
// (coherence_vector_representation.hpp:52-93): u_jk, then v_jk, then w_l.
MBG_HD int generator_entries(int N, int i, int* r, int* c, cd* v)
{
    int P = N * (N - 1) / 2;
    if (i < 2 * P) {
        int p = (i < P) ? i : i - P;
        int k = 1;
        while (k * (k + 1) / 2 <= p) k++;
        int j = p - k * (k - 1) / 2;
        r[0] = j;
        c[0] = k;
        r[1] = k;
        c[1] = j;
        if (i < P) {
            v[0] = cmake(1, 0);
            v[1] = cmake(1, 0);
        } else {
            v[0] = cmake(0, -1);
            v[1] = cmake(0, 1);
        }
        return 2;
    }
    int l = i - 2 * P;
    double nrm = 1.0 / sqrt((double) (((l + 1) * (l + 2)) / 2));
    int cnt = 0;
    for (int j = 0; j <= l; j++) {
        r[cnt] = j;
        c[cnt] = j;
        v[cnt] = cmake(-nrm, 0);
        cnt++;
    }
    r[cnt] = l + 1;
    c[cnt] = l + 1;
    v[cnt] = cmake((l + 1) * nrm, 0);
    return cnt + 1;
}

// tr(A g) for dense A (N x N complex) and sparse generator g
MBG_HD cd trace_with_gen(
    const double* are,
    const double* aim,
    int N,
    int nz,
    const int* r,
    const int* c,
    const cd* v)
{
    cd s = cmake(0, 0);
    for (int e = 0; e < nz; e++) {
        cd a = cmake(are[c[e] * N + r[e]], aim[c[e] * N + r[e]]);
        s = cadd(s, cmul(a, v[e]));
    }
    return s;
}

// Lindblad relaxation action on a Hermitian matrix (qm_description.hpp:
// 211-236); the base superoperator (relax_kind 0) returns zero.
MBG_HD void relax_apply(
    const mat_in& m,
    const double* xre,
    const double* xim,
    double* yre,
    double* yim)
{
    int N = m.N;
    for (int i = 0; i < N * N; i++) yre[i] = yim[i] = 0.0;
    if (m.relax_kind != 1) return;
    for (int a = 0; a < N; a++) {
        double s = 0.0;
        for (int b = 0; b < N; b++) s += m.S[a * N + b] * xre[b * N + b];
        yre[a * N + a] = s;
    }
    for (int k = 1; k < N; k++)
        for (int j = 0; j < k; j++) {
            double d = m.deph[upper_index(j, k)];
            double zr = xre[j * N + k] * d, zi = xim[j * N + k] * d;
            yre[j * N + k] = zr;
            yim[j * N + k] = zi;
            yre[k * N + j] = zr;
            yim[k * N + j] = -zi;
        }
}

// Coherence vector of the initial density matrix exactly as
// coherence_vector_representation.hpp:341-394 computes it (including its
// indexing: every off-diagonal entry writes the first slot of its block,
// so only the last entry's value is kept there).
MBG_HD void initial_coherence_vector(const mat_in& m, double* d)
{
    int N = m.N, V = N * N - 1, P = N * (N - 1) / 2;
    for (int i = 0; i < V; i++) d[i] = 0.0;
    int rn = m.rho_levels;
    int rp = m.rho_num_off;
    for (int j = 0; j < rp; j++) d[0] = 2 * m.rho_off_re[j];
    for (int j = 0; j < rp; j++) d[P] = -2 * m.rho_off_im[j];
    for (int l = 0; l < N - 1; l++) {
        double e = 0.0;
        int j = 0;
        for (j = 0; j <= l; j++) e += -1.0 * (j < rn ? m.rho_diag[j] : 0.0);
        e += (l + 1) * (j < rn ? m.rho_diag[j] : 0.0);
        d[2 * P + l] = e / sqrt((double) (((l + 1) * (l + 2)) / 2));
    }
}

// Population weights of coherence_vector_representation.hpp:289-336:
// rho_mm = 1/N + 1/2 sum_i w_i d[N(N-1) + i].
MBG_HD double population_weight(int N, int m, int i)
{
    if (N == 3 && m > 2) return 0.0;
    double f;
    if (m < i + 1)
        f = -1.0;
    else if (m == i + 1)
        f = (double) m;
    else
        f = 0.0;
    return f / sqrt((double) (((i + 1) * (i + 2)) / 2));
}
MBG_HD double population_const(int N, int m)
{
    return (N == 3 && m > 2) ? 0.0 : 1.0 / N;
}

// Workspace doubles needed by cvr_precompute for N levels.
MBG_HD size_t cvr_workspace(int N)
{
    size_t V = (size_t) N * N - 1;
    return V * N * N * 2 + V * V * 14 + V * 12 + 64;
}

// FDTD constants (common_fdtd.hpp:158-190).
MBG_HD void fdtd_constants(const mat_in& m, double* a, double* b, double* c)
{
    double sigma = sqrt(EPS0 * m.eps_r / (MU0 * m.mu_r)) * m.losses * 2.0;
    double epsilon = EPS0 * m.eps_r;
    double x = (sigma * m.dt) / (2.0 * epsilon);
    *a = (1.0 - x) / (1.0 + x);
    *b = m.dt / epsilon / (1.0 + x);
    *c = m.dt / (MU0 * m.mu_r * m.dx);
}

// The FDTD entries of a material block (see FD_* above).
MBG_HD void write_fdtd(const mat_in& m, double* out)
{
    double a, b, c;
    fdtd_constants(m, &a, &b, &c);
    out[FD_A] = a;
    out[FD_B] = b;
    out[FD_C] = c;
    out[FD_GAMMA] = m.overlap;
    const double bdx = b / m.dx;
    out[FD_BDX] = bdx;
    out[FD_BDX_LO] = bdx - (double) (float) bdx;
    out[FD_C_LO] = c - (double) (float) c;
    out[FD_G] = b * m.overlap;
}

// Coherence-vector constants of one material into out (cvr_layout of
// `Nsolver` levels). Returns 0 on success, 1 when the level count does not
// match the solver, 2 when M d_in = d_eq has no solution (the reference's
// "Time-indepent matrix not invertible!" check, rodr.hpp:195-206).
MBG_HD int cvr_precompute(const mat_in& m, int Nsolver, double* ws, double* out)
{
    cvr_layout L = make_cvr_layout(Nsolver);
    for (int i = 0; i < L.stride; i++) out[i] = 0.0;
    write_fdtd(m, out);
    const int N = Nsolver, V = L.V, KP = L.KP;
    if (m.N == 0) {
        // no quantum-mechanical description: the density stays the zero
        // vector, whose populations are 1/N (cvr.hpp:289-336)
        out[L.has_qm] = 0.0;
        for (int k = 0; k < N; k++) out[L.pop_c + k] = population_const(N, k);
        return 0;
    }
    if (m.N != Nsolver) return 1;
    out[L.has_qm] = 1.0;
    const int NN = N * N;
    double* X = ws;                        // V * N*N * 2 : op * g_i
    double* Tr = X + (size_t) V * NN * 2;  // V*V*2 : tr(op g_i g_j)
    double* M = Tr + V * V * 2;
    double* U = M + V * V;
    double* F = U + V * V;
    double* Q = F + V * V;
    double* H1 = Q + V * V;   // Hermitian re
    double* H2 = H1 + V * V;  // Hermitian im
    double* E1 = H2 + V * V;  // eigvec re
    double* E2 = E1 + V * V;  // eigvec im
    double* W = E2 + V * V;   // 3 V*V expm workspace
    double* vec = W + 3 * V * V;
    double* v_dip = vec;
    double* d_eq = vec + V;
    double* d_in = vec + 2 * V;
    double* t1 = vec + 3 * V;
    double* t2 = vec + 4 * V;
    double* lam = vec + 5 * V;
    double* d0 = vec + 6 * V;
    double* tre = vec + 7 * V;  // N*N (<= V+1)
    double* tim = tre + NN;
    double* ure = tim + NN;
    double* uim = ure + NN;

    int gr[8], gc[8];
    cd gv[8];
    // Liouvillians L(op)_ij = Re(i/2 tr(op [g_i, g_j])) / hbar
    // (coherence_vector_representation.hpp:149-166) of H and mu
    for (int which = 0; which < 2; which++) {
        const double* ore = which == 0 ? m.h_re : m.mu_re;
        const double* oim = which == 0 ? m.h_im : m.mu_im;
        for (int i = 0; i < V; i++) {
            int nz = generator_entries(N, i, gr, gc, gv);
            double* xr = X + (size_t) i * NN * 2;
            double* xi = xr + NN;
            for (int e = 0; e < NN; e++) xr[e] = xi[e] = 0.0;
            // (op g)(r', c) = sum over entries g(r, c): op(r', r) g(r, c)
            for (int e = 0; e < nz; e++)
                for (int rr = 0; rr < N; rr++) {
                    cd o = cmake(ore[rr * N + gr[e]], oim[rr * N + gr[e]]);
                    cd p = cmul(o, gv[e]);
                    xr[rr * N + gc[e]] += p.re;
                    xi[rr * N + gc[e]] += p.im;
                }
        }
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                int nz = generator_entries(N, j, gr, gc, gv);
                const double* xr = X + (size_t) i * NN * 2;
                cd t = trace_with_gen(xr, xr + NN, N, nz, gr, gc, gv);
                Tr[(i * V + j) * 2] = t.re;
                Tr[(i * V + j) * 2 + 1] = t.im;
            }
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                double dim = Tr[(i * V + j) * 2 + 1] - Tr[(j * V + i) * 2 + 1];
                double l = -0.5 * dim / HBAR;  // Re(i z / 2) = -Im(z) / 2
                if (which == 0)
                    M[i * V + j] = l;
                else
                    U[i * V + j] = -l;  // U = -L(mu)
            }
        if (which == 1) {
            // dipole vector v_i = Re tr(mu g_i) (cvr.hpp:168-179)
            for (int i = 0; i < V; i++) {
                int nz = generator_entries(N, i, gr, gc, gv);
                v_dip[i] = trace_with_gen(m.mu_re, m.mu_im, N, nz, gr, gc, gv).re;
            }
        }
    }
    // relaxation superoperator G_ij = Re 1/2 tr(R(g_j) g_i) and the
    // equilibrium vector d_eq_i = Re tr(R(I) g_i) / N (cvr.hpp:181-213)
    for (int j = 0; j < V; j++) {
        int nz = generator_entries(N, j, gr, gc, gv);
        for (int e = 0; e < NN; e++) tre[e] = tim[e] = 0.0;
        for (int e = 0; e < nz; e++) {
            tre[gr[e] * N + gc[e]] = gv[e].re;
            tim[gr[e] * N + gc[e]] = gv[e].im;
        }
        relax_apply(m, tre, tim, ure, uim);
        for (int i = 0; i < V; i++) {
            int nzi = generator_entries(N, i, gr, gc, gv);
            cd t = trace_with_gen(ure, uim, N, nzi, gr, gc, gv);
            M[i * V + j] += 0.5 * t.re;
        }
    }
    for (int e = 0; e < NN; e++) {
        tre[e] = (e % (N + 1) == 0) ? 1.0 : 0.0;
        tim[e] = 0.0;
    }
    relax_apply(m, tre, tim, ure, uim);
    for (int i = 0; i < V; i++) {
        int nz = generator_entries(N, i, gr, gc, gv);
        d_eq[i] = trace_with_gen(ure, uim, N, nz, gr, gc, gv).re / N;
    }
    const double M_CP = 0.5 * m.carrier_density;

    // d_in: M d_in = d_eq unless d_eq is zero (rodr.hpp:193-206)
    bool zero = true;
    for (int i = 0; i < V; i++)
        if (fabs(d_eq[i]) > 2.220446049250313e-16) zero = false;
    if (zero) {
        for (int i = 0; i < V; i++) d_in[i] = 0.0;
    } else {
        for (int i = 0; i < V * V; i++) F[i] = M[i];
        for (int i = 0; i < V; i++) t1[i] = d_eq[i];
        solve_partial_pivot(F, t1, d_in, V);
        double nr = 0.0, nd = 0.0;
        for (int i = 0; i < V; i++) {
            double s = -d_eq[i];
            for (int j = 0; j < V; j++) s += M[i * V + j] * d_in[j];
            nr += s * s;
            nd += d_eq[i] * d_eq[i];
        }
        if (!(sqrt(nr) / sqrt(nd) <= 1e-3)) return 2;
    }

    // F = exp(M dt/2) - I
    for (int i = 0; i < V * V; i++) H1[i] = M[i] * m.dt / 2;
    expm_minus_identity(H1, F, V, W);

    // planes of U from the Hermitian matrix i U
    for (int i = 0; i < V * V; i++) {
        H1[i] = 0.0;
        H2[i] = U[i];
    }
    jacobi_hermitian(H1, H2, E1, E2, V);
    for (int i = 0; i < V; i++) lam[i] = H1[i * V + i];
    double lmax = 0.0;
    for (int i = 0; i < V; i++) lmax = lam[i] > lmax ? lam[i] : lmax;
    int used[64];
    for (int i = 0; i < V; i++) used[i] = 0;
    int ncol = 0, nplanes = 0;
    while (nplanes < KP) {
        int best = -1;
        for (int i = 0; i < V; i++)
            if (!used[i] && lam[i] > 1e-9 * lmax && lmax > 0.0 &&
                (best < 0 || lam[i] > lam[best]))
                best = i;
        if (best < 0) break;
        used[best] = 1;
        // q1, q2 from the real and imaginary parts, re-orthonormalised
        double n1 = 0.0;
        for (int i = 0; i < V; i++) {
            t1[i] = E1[i * V + best];
            t2[i] = E2[i * V + best];
        }
        for (int pass = 0; pass < 2; pass++)
            for (int col = 0; col < ncol; col++) {
                double d1 = 0.0, d2 = 0.0;
                for (int i = 0; i < V; i++) {
                    d1 += Q[i * V + col] * t1[i];
                    d2 += Q[i * V + col] * t2[i];
                }
                for (int i = 0; i < V; i++) {
                    t1[i] -= d1 * Q[i * V + col];
                    t2[i] -= d2 * Q[i * V + col];
                }
            }
        for (int i = 0; i < V; i++) n1 += t1[i] * t1[i];
        n1 = sqrt(n1);
        if (n1 < 1e-3) continue;
        for (int i = 0; i < V; i++) t1[i] /= n1;
        double dd = 0.0;
        for (int i = 0; i < V; i++) dd += t1[i] * t2[i];
        double n2 = 0.0;
        for (int i = 0; i < V; i++) {
            t2[i] -= dd * t1[i];
            n2 += t2[i] * t2[i];
        }
        n2 = sqrt(n2);
        if (n2 < 1e-3) continue;
        for (int i = 0; i < V; i++) t2[i] /= n2;
        // theta = q2 . U q1 ; orient so that theta > 0
        double th = 0.0;
        for (int i = 0; i < V; i++) {
            double s = 0.0;
            for (int j = 0; j < V; j++) s += U[i * V + j] * t1[j];
            th += t2[i] * s;
        }
        if (th < 0) {
            th = -th;
            for (int i = 0; i < V; i++) t2[i] = -t2[i];
        }
        for (int i = 0; i < V; i++) {
            Q[i * V + ncol] = t1[i];
            Q[i * V + ncol + 1] = t2[i];
        }
        out[L.thdt + nplanes] = th * m.dt;
        ncol += 2;
        nplanes++;
    }
    out[L.nplanes] = nplanes;
    // complete Q with an orthonormal basis of the null space of U
    while (ncol < V) {
        int best = -1;
        double bestn = -1.0;
        for (int i = 0; i < V; i++) {
            double s = 1.0;
            for (int col = 0; col < ncol; col++)
                s -= Q[i * V + col] * Q[i * V + col];
            if (s > bestn) {
                bestn = s;
                best = i;
            }
        }
        for (int i = 0; i < V; i++) t1[i] = (i == best) ? 1.0 : 0.0;
        for (int pass = 0; pass < 2; pass++)
            for (int col = 0; col < ncol; col++) {
                double d = 0.0;
                for (int i = 0; i < V; i++) d += Q[i * V + col] * t1[i];
                for (int i = 0; i < V; i++) t1[i] -= d * Q[i * V + col];
            }
        double nn = 0.0;
        for (int i = 0; i < V; i++) nn += t1[i] * t1[i];
        nn = sqrt(nn);
        for (int i = 0; i < V; i++) Q[i * V + ncol] = t1[i] / nn;
        ncol++;
    }

    for (int i = 0; i < V * V; i++) out[L.Q + i] = Q[i];
    // out[o] = Q^T X Q for X (V x V, original basis); H1 is scratch
    auto to_planes = [&](const double* X, double* dst) {
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                double s = 0.0;
                for (int k = 0; k < V; k++) s += X[i * V + k] * Q[k * V + j];
                H1[i * V + j] = s;  // X Q
            }
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                double s = 0.0;
                for (int k = 0; k < V; k++) s += Q[k * V + i] * H1[k * V + j];
                dst[i * V + j] = s;
            }
    };
    // Q^T X d_in
    auto drive = [&](const double* X, double* dst) {
        for (int i = 0; i < V; i++) {
            double s = 0.0;
            for (int j = 0; j < V; j++) s += X[i * V + j] * d_in[j];
            t2[i] = s;
        }
        for (int k = 0; k < V; k++) {
            double s = 0.0;
            for (int i = 0; i < V; i++) s += Q[i * V + k] * t2[i];
            dst[k] = s;
        }
    };
    // half step: Bh = Q^T (exp(M dt/2) - I) Q, kh = Q^T (exp(M dt/2) - I) d_in
    double* Bh = out + L.Bh;
    double* kh = out + L.kh;
    to_planes(F, Bh);
    drive(F, kh);
    // full step: Bd = Q^T (exp(M dt) - I) Q, k = Q^T (exp(M dt) - I) d_in
    for (int i = 0; i < V * V; i++) H2[i] = M[i] * m.dt;
    expm_minus_identity(H2, E1, V, W);
    to_planes(E1, out + L.Bd);
    for (int i = 0; i < V * V; i++) out[L.Bdl + i] = out[L.Bd + i] - (double) (float) out[L.Bd + i];
    drive(E1, out + L.k);
    // Bi = A^-1 - I = Q^T (exp(-M dt/2) - I) Q
    for (int i = 0; i < V * V; i++) H2[i] = -M[i] * m.dt / 2;
    expm_minus_identity(H2, E2, V, W);
    double* Bi = E1;
    to_planes(E2, Bi);
    // a row r on u becomes r (I + Bi) on v with constant -r (I + Bi) kh
    auto compose = [&](double* r, double& c) {
        for (int j = 0; j < V; j++) {
            double s = r[j];
            for (int i = 0; i < V; i++) s += r[i] * Bi[i * V + j];
            t1[j] = s;
        }
        for (int j = 0; j < V; j++) {
            r[j] = t1[j];
            c -= t1[j] * kh[j];
        }
    };
    // P = p0 + g . u with g = M_CP Q^T M^T v_dip, p0 = M_CP v_dip . d_eq
    // (rodr.hpp:258-266)
    for (int j = 0; j < V; j++) {
        double s = 0.0;
        for (int i = 0; i < V; i++) s += M[i * V + j] * v_dip[i];
        t2[j] = s;  // (M^T v)_j
    }
    double p0 = 0.0;
    for (int i = 0; i < V; i++) p0 += v_dip[i] * d_eq[i];
    for (int k = 0; k < V; k++) {
        double sg = 0.0;
        for (int i = 0; i < V; i++) sg += Q[i * V + k] * t2[i];
        out[L.g + k] = M_CP * sg;
    }
    p0 *= M_CP;
    compose(out + L.g, p0);
    out[L.p0] = p0;
    // initial state v0 = A u0 + kh, u0 = Q^T d0
    initial_coherence_vector(m, d0);
    for (int k = 0; k < V; k++) {
        double s = 0.0;
        for (int i = 0; i < V; i++) s += Q[i * V + k] * d0[i];
        t2[k] = s;
    }
    for (int i = 0; i < V; i++) {
        double s = t2[i] + kh[i];
        for (int j = 0; j < V; j++) s += Bh[i * V + j] * t2[j];
        out[L.z0 + i] = s;
    }
    // observables: d = Q u
    int w0 = N * (N - 1);
    for (int k = 0; k < V; k++) out[L.inv + k] = Q[w0 * V + k];
    out[L.inv_c] = 0.0;
    compose(out + L.inv, out[L.inv_c]);
    for (int mm = 0; mm < N; mm++) {
        for (int k = 0; k < V; k++) out[L.pop + mm * V + k] = 0.0;
        for (int i = 0; i < N - 1; i++) {
            double w = 0.5 * population_weight(N, mm, i);
            for (int k = 0; k < V; k++)
                out[L.pop + mm * V + k] += w * Q[(w0 + i) * V + k];
        }
        out[L.pop_c + mm] = population_const(N, mm);
        compose(out + L.pop + mm * V, out[L.pop_c + mm]);
    }
    // coherences: rho = I/N + 1/2 sum_i d_i g_i, so rho[j][k] (j != k) is
    // 1/2 sum_i (g_i)[j][k] d_i: real and imaginary rows on d, then on u
    // (d = Q u), then composed with A1^-1 like the other records
    for (int kk = 1; kk < N; kk++)
        for (int jj = 0; jj < kk; jj++) {
            const int q = kk * (kk - 1) / 2 + jj;
            for (int part = 0; part < 2; part++) {
                for (int i = 0; i < V; i++) t2[i] = 0.0;
                for (int i = 0; i < V; i++) {
                    int nz = generator_entries(N, i, gr, gc, gv);
                    for (int e = 0; e < nz; e++)
                        if (gr[e] == jj && gc[e] == kk) t2[i] += 0.5 * (part == 0 ? gv[e].re : gv[e].im);
                }
                double* row = out + L.coh + (2 * q + part) * V;
                for (int c = 0; c < V; c++) {
                    double s = 0.0;
                    for (int i = 0; i < V; i++) s += t2[i] * Q[i * V + c];
                    row[c] = s;
                }
                out[L.coh_c + 2 * q + part] = 0.0;
                compose(row, out[L.coh_c + 2 * q + part]);
            }
        }
    return 0;
}

// Workspace doubles needed by cay_precompute.
MBG_HD size_t cay_workspace(int N) { return (size_t) N * N * 18 + 16; }

MBG_HD void pack_hermitian(const double* re, const double* im, int N, double s, double* out)
{
    for (int i = 0; i < N; i++) out[i] = re[i * N + i] * s;
    for (int k = 1; k < N; k++)
        for (int j = 0; j < k; j++) {
            int p = upper_index(j, k);
            out[N + 2 * p] = re[j * N + k] * s;
            out[N + 2 * p + 1] = im[j * N + k] * s;
        }
}

// Entry (j, k) of a Hermitian matrix stored packed (diagonal, then the upper
// triangle column-major as (re, im) pairs).
MBG_HD void herm_at(const double* p, int N, int j, int k, double& re, double& im)
{
    if (j == k) {
        re = p[j];
        im = 0.0;
    } else if (j < k) {
        const int q = upper_index(j, k);
        re = p[N + 2 * q];
        im = p[N + 2 * q + 1];
    } else {
        const int q = upper_index(k, j);
        re = p[N + 2 * q];
        im = -p[N + 2 * q + 1];
    }
}

// The polarisation current of the Cayley update (reg_cayley.hpp:258-267),
// P = Re tr((-i [W0, rho] + D'(rho)) Mn), is real-linear in the packed
// density matrix r: P = gP . r. With C = Mn W0 - W0 Mn (anti-Hermitian),
// Re tr(-i [W0, rho] Mn) = Im tr(rho C), and for r's coordinates
//   diagonal l:        Im C_ll + sum_j d1[j][l] Mn_jj
//   Re rho_jk (j < k): 2 Im C_jk + 2 gamma_jk Re Mn_jk
//   Im rho_jk (j < k): -2 Re C_jk + 2 gamma_jk Im Mn_jk
// (gamma_jk the dephasing rate of the pair, D'(rho)_jk = gamma_jk rho_jk).
// Evaluated per material in FP64; the kernels then need N^2 FMAs per point.
MBG_HD void cay_polarisation_weights(const cay_layout& L, double* out)
{
    const int N = L.N;
    const double* W = out + L.W0;
    const double* Mn = out + L.Mn;
    for (int j = 0; j < N; j++)
        for (int k = j; k < N; k++) {
            // C_jk = sum_l Mn_jl W_lk - W_jl Mn_lk
            double cr = 0.0, ci = 0.0;
            for (int l = 0; l < N; l++) {
                double mr, mi, wr, wi;
                herm_at(Mn, N, j, l, mr, mi);
                herm_at(W, N, l, k, wr, wi);
                cr += mr * wr - mi * wi;
                ci += mr * wi + mi * wr;
                herm_at(W, N, j, l, wr, wi);
                herm_at(Mn, N, l, k, mr, mi);
                cr -= wr * mr - wi * mi;
                ci -= wr * mi + wi * mr;
            }
            if (j == k) {
                double s = ci;
                for (int i = 0; i < N; i++) s += out[L.d1 + i * N + j] * Mn[i];
                out[L.gP + j] = s;
            } else {
                const int q = upper_index(j, k);
                const double g2 = out[L.d2 + q];
                out[L.gP + N + 2 * q] = 2.0 * ci + 2.0 * g2 * Mn[N + 2 * q];
                out[L.gP + N + 2 * q + 1] = -2.0 * cr + 2.0 * g2 * Mn[N + 2 * q + 1];
            }
        }
}

// Solves A X = B for n x n complex A and n x m complex B (row-major; A and B
// are overwritten, X is left in B) by Gaussian elimination with partial
// pivoting on the modulus.
MBG_HD void csolve(cd* A, cd* B, int n, int m)
{
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = A[k * n + k].re * A[k * n + k].re + A[k * n + k].im * A[k * n + k].im;
        for (int i = k + 1; i < n; i++) {
            const double v = A[i * n + k].re * A[i * n + k].re + A[i * n + k].im * A[i * n + k].im;
            if (v > best) {
                best = v;
                p = i;
            }
        }
        if (p != k) {
            for (int j = 0; j < n; j++) {
                const cd t = A[k * n + j];
                A[k * n + j] = A[p * n + j];
                A[p * n + j] = t;
            }
            for (int j = 0; j < m; j++) {
                const cd t = B[k * m + j];
                B[k * m + j] = B[p * m + j];
                B[p * m + j] = t;
            }
        }
        const cd piv = A[k * n + k];
        const double den = piv.re * piv.re + piv.im * piv.im;
        const cd inv = cmake(piv.re / den, -piv.im / den);
        for (int i = k + 1; i < n; i++) {
            const cd f = cmul(A[i * n + k], inv);
            for (int j = k; j < n; j++) A[i * n + j] = csub(A[i * n + j], cmul(f, A[k * n + j]));
            for (int j = 0; j < m; j++) B[i * m + j] = csub(B[i * m + j], cmul(f, B[k * m + j]));
        }
    }
    for (int k = n - 1; k >= 0; k--) {
        const cd piv = A[k * n + k];
        const double den = piv.re * piv.re + piv.im * piv.im;
        const cd inv = cmake(piv.re / den, -piv.im / den);
        for (int j = 0; j < m; j++) {
            cd s = B[k * m + j];
            for (int i = k + 1; i < n; i++) s = csub(s, cmul(A[k * n + i], B[i * m + j]));
            B[k * m + j] = cmul(s, inv);
        }
    }
}

// Full Hermitian matrix (n x n, row-major) from its packed form, and back.
MBG_HD void herm_unpack(const double* p, int N, cd* F)
{
    for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) herm_at(p, N, j, k, F[j * N + k].re, F[j * N + k].im);
}
MBG_HD void herm_pack(const cd* F, int N, double* p)
{
    for (int i = 0; i < N; i++) p[i] = F[i * N + i].re;
    for (int k = 1; k < N; k++)
        for (int j = 0; j < k; j++) {
            const int q = upper_index(j, k);
            p[N + 2 * q] = F[j * N + k].re;
            p[N + 2 * q + 1] = F[j * N + k].im;
        }
}

// (D - I) r for the dissipation half step D on a packed density matrix:
// populations by D1 - I, the coherence of pair q by D2_q - 1.
MBG_HD void cay_dissipation_increment(const cay_layout& L, const double* out, const double* r, double* d)
{
    const int N = L.N;
    for (int i = 0; i < N; i++) {
        double s = 0.0;
        for (int j = 0; j < N; j++) s += out[L.dD1 + i * N + j] * r[j];
        d[i] = s;
    }
    for (int q = 0; q < L.P; q++) {
        d[N + 2 * q] = out[L.dD2 + q] * r[N + 2 * q];
        d[N + 2 * q + 1] = out[L.dD2 + q] * r[N + 2 * q + 1];
    }
}

// The field-free part of the FP32 Cayley step (see cay_layout): U0, W and
// B0 = D Ad(U0) D - I from kH0, kMu, dD1 and dD2, all in FP64. B0's
// columns are formed as sums of small increments (never as T0 e - e), so
// its entries keep their relative accuracy however small the rates. With
// a diagonal H0 (every preset but the random media) U0 is diagonal and B0
// block-diagonal, exactly: populations mix among themselves, each
// coherence (re, im) only with itself; blockB0 = 1 lets the kernels skip
// the zero blocks (the same sums without exact zero terms).
// ws: 17 N^2 doubles.
MBG_HD void cay_free_step(const cay_layout& L, double* ws, double* out)
{
    const int N = L.N, NN = N * N;
    cd* A = reinterpret_cast<cd*>(ws);  // NN
    cd* B = A + NN;                      // N x 2N: [Y | A0^-1]
    cd* X = B + 2 * NN;                  // X0 = U0 - I
    cd* K = X + NN;                      // K1, then scratch
    cd* S = K + NN;                      // sigma (full)
    cd* G = S + NN;                      // X0 sigma
    double* r = reinterpret_cast<double*>(G + NN);  // NN packed
    double* t = r + NN;
    double* d = t + NN;
    // A0 = I + i K0; solve A0 [Y | Ai] = [K0 | I]
    for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) {
            double kr, ki;
            herm_at(out + L.kH0, N, j, k, kr, ki);
            A[j * N + k] = cmake((j == k ? 1.0 : 0.0) - ki, kr);
            B[j * 2 * N + k] = cmake(kr, ki);
            B[j * 2 * N + N + k] = cmake(j == k ? 1.0 : 0.0, 0.0);
        }
    csolve(A, B, N, 2 * N);
    // X0 = -2i Y; U0 = I + X0
    for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) {
            const cd y = B[j * 2 * N + k];
            X[j * N + k] = cmake(2.0 * y.im, -2.0 * y.re);
            out[L.U0 + j * N + k] = (j == k ? 1.0 : 0.0) + X[j * N + k].re;
            out[L.U0 + NN + j * N + k] = X[j * N + k].im;
        }
    // W = K1 A0^-1
    for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) {
            double kr, ki;
            herm_at(out + L.kMu, N, j, k, kr, ki);
            K[j * N + k] = cmake(kr, ki);
        }
    for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) {
            cd s = cmake(0.0, 0.0);
            for (int l = 0; l < N; l++) s = cadd(s, cmul(K[j * N + l], B[l * 2 * N + N + k]));
            out[L.Wk + j * N + k] = s.re;
            out[L.Wk + NN + j * N + k] = s.im;
        }
    bool diag = true;
    for (int q = 0; q < L.P; q++)
        if (out[L.kH0 + N + 2 * q] != 0.0 || out[L.kH0 + N + 2 * q + 1] != 0.0) diag = false;
    out[L.blockB0] = diag ? 1.0 : 0.0;
    // columns of B0: e_v -> (D - I) e_v + pack(Ad(U0) s - s) + (D - I) tau,
    // s = D e_v, tau = Ad(U0) s
    for (int v = 0; v < NN; v++) {
        for (int i = 0; i < NN; i++) r[i] = (i == v) ? 1.0 : 0.0;
        cay_dissipation_increment(L, out, r, d);  // (D - I) e_v
        for (int i = 0; i < NN; i++) t[i] = r[i] + d[i];
        herm_unpack(t, N, S);
        // Ad(U0) s - s = X0 s + (X0 s)^H + X0 s X0^H
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                cd g = cmake(0.0, 0.0);
                for (int l = 0; l < N; l++) g = cadd(g, cmul(X[j * N + l], S[l * N + k]));
                G[j * N + k] = g;
            }
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                cd h = cadd(G[j * N + k], cconj(G[k * N + j]));
                for (int l = 0; l < N; l++) h = cadd(h, cmul(G[j * N + l], cconj(X[k * N + l])));
                K[j * N + k] = h;
            }
        herm_pack(K, N, r);  // Ad(U0) s - s, packed
        for (int i = 0; i < NN; i++) {
            d[i] += r[i];       // column so far: (D - I) e_v + (Ad(U0) s - s)
            t[i] += r[i];       // tau = s + (Ad(U0) s - s)
        }
        cay_dissipation_increment(L, out, t, r);  // (D - I) tau
        for (int i = 0; i < NN; i++) {
            const double b = d[i] + r[i];
            out[L.B0 + i * L.NP + v] = b;
            out[L.B0l + i * L.NP + v] = b - (double) (float) b;
        }
    }
}

// Cayley constants of one material (cay_layout of `Nsolver` levels).
// Returns 0, 1 on a level-count mismatch, 3 for a relaxation superoperator
// that is not of Lindblad form (reg_cayley.hpp:146-155).
MBG_HD int cay_precompute(const mat_in& m, int Nsolver, double* ws, double* out)
{
    cay_layout L = make_cay_layout(Nsolver);
    for (int i = 0; i < L.stride; i++) out[i] = 0.0;
    write_fdtd(m, out);
    int N = Nsolver;
    if (m.N == 0) {
        out[L.has_qm] = 0.0;
        return 0;
    }
    if (m.N != Nsolver) return 1;
    if (m.relax_kind != 1) return 3;
    out[L.has_qm] = 1.0;
    const double kappa = m.dt / (2.0 * HBAR);
    pack_hermitian(m.h_re, m.h_im, N, kappa, out + L.kH0);
    pack_hermitian(m.mu_re, m.mu_im, N, kappa, out + L.kMu);
    pack_hermitian(m.h_re, m.h_im, N, 1.0 / HBAR, out + L.W0);
    pack_hermitian(m.mu_re, m.mu_im, N, m.carrier_density, out + L.Mn);
    double* X = ws;
    double* Fm = ws + N * N;
    double* W = ws + 2 * N * N;
    for (int i = 0; i < N * N; i++) X[i] = m.S[i] * m.dt / 2;
    expm_minus_identity(X, Fm, N, W);
    for (int i = 0; i < N * N; i++) {
        out[L.dD1 + i] = Fm[i];
        out[L.d1 + i] = m.S[i];
    }
    for (int p = 0; p < L.P; p++) {
        out[L.dD2 + p] = expm1(m.deph[p] * m.dt / 2);
        out[L.d2 + p] = m.deph[p];
    }
    // initial density matrix (reg_cayley.hpp:269-272)
    int rn = m.rho_levels;
    for (int i = 0; i < N; i++) out[L.rho0 + i] = i < rn ? m.rho_diag[i] : 0.0;
    for (int p = 0; p < L.P && p < m.rho_num_off; p++) {
        out[L.rho0 + N + 2 * p] = m.rho_off_re[p];
        out[L.rho0 + N + 2 * p + 1] = m.rho_off_im[p];
    }
    cay_polarisation_weights(L, out);
    cay_free_step(L, ws, out);
    return 0;
}

// FDTD-only constants (Maxwell solver, algo_lindblad_noop.hpp)
MBG_HD int noop_precompute(const mat_in& m, double* out)
{
    cvr_layout L = make_cvr_layout(0);
    for (int i = 0; i < L.stride; i++) out[i] = 0.0;
    write_fdtd(m, out);
    return 0;
}

}  // namespace pre
}  // namespace mbg
