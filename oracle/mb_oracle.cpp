/*
 * ORACLE — test infrastructure only.
 *
 * A CPU, FP64 restatement of mbsolve's plain FDTD time loop and of its two
 * Lindblad propagators, used to check the GPU engine. Nothing in the
 * product links, imports or calls this file; only the tests, the smoke
 * check and the benchmark's CPU-baseline leg do.
 *
 * It follows, function by function (paths relative to the mbsolve tree):
 *   types.hpp:36-73                      physical constants
 *   internal/common_fdtd.hpp:52-123      init_fdtd_simulation
 *   internal/common_fdtd.hpp:158-190     get_fdtd_constants
 *   internal/coherence_vector_representation.hpp:52-394   SU(N) CVR
 *   internal/algo_lindblad_cvr_rodr.hpp:101-299  Rodrigues propagator
 *   internal/algo_lindblad_reg_cayley.hpp:91-274 Cayley propagator
 *   internal/algo_lindblad_noop.hpp:35-86        Maxwell only
 *   internal/copy_list_entry.hpp:51-229  recording plan
 *   solver-cpu/.../solver_cpu_fdtd.tpp:36-338    constructor and run()
 *   solver-cpu/.../solver_cpu_fdtd_red.tpp:351-567  the temporally blocked
 *                                        loop (run_red; same results)
 *   qm_description.hpp:166-236           Lindblad relaxation action
 *   source.hpp:94-106,190-194,256-260    source waveforms
 * The reference leans on Eigen for three numerical kernels; this file has
 * its own versions of them, each a named published method:
 *   matrix exponential: scaling and squaring with Pade approximants of
 *     degree 3/5/7/9/13 (N. J. Higham, SIAM J. Matrix Anal. Appl. 26(4),
 *     2005), in place of Eigen's MatrixFunctions exp();
 *   real Schur planes of the skew-symmetric dipole Liouvillian: cyclic
 *     Jacobi eigen-decomposition of the symmetric U^T U (Golub & Van Loan,
 *     Matrix Computations, 4th ed., sec. 8.5), then pairing q2 = U q1/theta,
 *     in place of Eigen::RealSchur;
 *   linear solves: Gaussian elimination with full pivoting (in place of
 *     FullPivLU) and Gauss-Jordan with partial pivoting (in place of
 *     inverse()).
 * Deliberate deviations from the reference: a soft source
 * is applied once per step (the reference applies it once per OpenMP
 * thread, solver_cpu_fdtd.tpp:245-255); the 2-level closed form guards
 * theta_1 = 0 (the reference divides by zero there).
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mbsolve_gb300.h"

namespace mbo {

typedef double real;
typedef std::complex<double> cplx;

/* types.hpp:36-73 */
static const real HBAR = 1.05457266e-34;
static const real PI = std::atan(1.0) * 4.0;
static const real MU0 = PI * 4e-7;
static const real EPS0 = 8.854187817e-12;

/* ------------------------------------------------------------ matrices */

struct rmat {
    int n = 0, m = 0;
    std::vector<real> a;
    rmat() {}
    rmat(int n_, int m_) : n(n_), m(m_), a((size_t) n_ * m_, 0.0) {}
    real& operator()(int i, int j) { return a[(size_t) i * m + j]; }
    real operator()(int i, int j) const { return a[(size_t) i * m + j]; }
    static rmat eye(int n_)
    {
        rmat r(n_, n_);
        for (int i = 0; i < n_; i++) r(i, i) = 1.0;
        return r;
    }
};

struct cmat {
    int n = 0;
    std::vector<cplx> a;
    cmat() {}
    explicit cmat(int n_) : n(n_), a((size_t) n_ * n_, cplx(0, 0)) {}
    cplx& operator()(int i, int j) { return a[(size_t) i * n + j]; }
    cplx operator()(int i, int j) const { return a[(size_t) i * n + j]; }
};

static rmat mul(const rmat& x, const rmat& y)
{
    rmat r(x.n, y.m);
    for (int i = 0; i < x.n; i++)
        for (int k = 0; k < x.m; k++) {
            real v = x(i, k);
            if (v == 0.0) continue;
            for (int j = 0; j < y.m; j++) r(i, j) += v * y(k, j);
        }
    return r;
}

static rmat add(const rmat& x, const rmat& y, real s = 1.0)
{
    rmat r = x;
    for (size_t i = 0; i < r.a.size(); i++) r.a[i] += s * y.a[i];
    return r;
}

static rmat scale(const rmat& x, real s)
{
    rmat r = x;
    for (auto& v : r.a) v *= s;
    return r;
}

static rmat transpose(const rmat& x)
{
    rmat r(x.m, x.n);
    for (int i = 0; i < x.n; i++)
        for (int j = 0; j < x.m; j++) r(j, i) = x(i, j);
    return r;
}

static std::vector<real> matvec(const rmat& x, const std::vector<real>& v)
{
    std::vector<real> r(x.n, 0.0);
    for (int i = 0; i < x.n; i++) {
        real s = 0.0;
        for (int j = 0; j < x.m; j++) s += x(i, j) * v[j];
        r[i] = s;
    }
    return r;
}

static cmat cmul(const cmat& x, const cmat& y)
{
    cmat r(x.n);
    for (int i = 0; i < x.n; i++)
        for (int k = 0; k < x.n; k++) {
            cplx v = x(i, k);
            for (int j = 0; j < x.n; j++) r(i, j) += v * y(k, j);
        }
    return r;
}

static cplx ctrace(const cmat& x)
{
    cplx t(0, 0);
    for (int i = 0; i < x.n; i++) t += x(i, i);
    return t;
}

/* Gaussian elimination with full pivoting: solves A x = b (A square). */
static std::vector<real> solve_full_pivot(rmat A, std::vector<real> b)
{
    int n = A.n;
    std::vector<int> colperm(n);
    std::iota(colperm.begin(), colperm.end(), 0);
    for (int k = 0; k < n; k++) {
        int pr = k, pc = k;
        real best = -1.0;
        for (int i = k; i < n; i++)
            for (int j = k; j < n; j++)
                if (std::fabs(A(i, j)) > best) {
                    best = std::fabs(A(i, j));
                    pr = i;
                    pc = j;
                }
        if (pr != k) {
            for (int j = 0; j < n; j++) std::swap(A(k, j), A(pr, j));
            std::swap(b[k], b[pr]);
        }
        if (pc != k) {
            for (int i = 0; i < n; i++) std::swap(A(i, k), A(i, pc));
            std::swap(colperm[k], colperm[pc]);
        }
        if (A(k, k) == 0.0) continue; /* singular block: leave zeros */
        for (int i = k + 1; i < n; i++) {
            real f = A(i, k) / A(k, k);
            if (f == 0.0) continue;
            for (int j = k; j < n; j++) A(i, j) -= f * A(k, j);
            b[i] -= f * b[k];
        }
    }
    std::vector<real> y(n, 0.0);
    for (int k = n - 1; k >= 0; k--) {
        if (A(k, k) == 0.0) {
            y[k] = 0.0;
            continue;
        }
        real s = b[k];
        for (int j = k + 1; j < n; j++) s -= A(k, j) * y[j];
        y[k] = s / A(k, k);
    }
    std::vector<real> x(n, 0.0);
    for (int k = 0; k < n; k++) x[colperm[k]] = y[k];
    return x;
}

/* Real inverse by Gauss-Jordan with partial pivoting. */
static rmat inverse(const rmat& A)
{
    int n = A.n;
    rmat a = A, r = rmat::eye(n);
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int i = k + 1; i < n; i++)
            if (std::fabs(a(i, k)) > std::fabs(a(p, k))) p = i;
        if (p != k)
            for (int j = 0; j < n; j++) {
                std::swap(a(k, j), a(p, j));
                std::swap(r(k, j), r(p, j));
            }
        real d = a(k, k);
        for (int j = 0; j < n; j++) {
            a(k, j) /= d;
            r(k, j) /= d;
        }
        for (int i = 0; i < n; i++) {
            if (i == k) continue;
            real f = a(i, k);
            if (f == 0.0) continue;
            for (int j = 0; j < n; j++) {
                a(i, j) -= f * a(k, j);
                r(i, j) -= f * r(k, j);
            }
        }
    }
    return r;
}

/* Complex inverse by Gauss-Jordan with partial pivoting. */
static cmat cinverse(const cmat& A)
{
    int n = A.n;
    cmat a = A, r(n);
    for (int i = 0; i < n; i++) r(i, i) = 1.0;
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int i = k + 1; i < n; i++)
            if (std::abs(a(i, k)) > std::abs(a(p, k))) p = i;
        if (p != k)
            for (int j = 0; j < n; j++) {
                std::swap(a(k, j), a(p, j));
                std::swap(r(k, j), r(p, j));
            }
        cplx d = a(k, k);
        for (int j = 0; j < n; j++) {
            a(k, j) /= d;
            r(k, j) /= d;
        }
        for (int i = 0; i < n; i++) {
            if (i == k) continue;
            cplx f = a(i, k);
            if (f == cplx(0, 0)) continue;
            for (int j = 0; j < n; j++) {
                a(i, j) -= f * a(k, j);
                r(i, j) -= f * r(k, j);
            }
        }
    }
    return r;
}

/* Matrix exponential: scaling and squaring with Pade approximants
 * (Higham 2005). Coefficients b_j = (2m-j)! m! / ((2m)! j! (m-j)!). */
static rmat expm(const rmat& A)
{
    int n = A.n;
    real norm1 = 0.0;
    for (int j = 0; j < n; j++) {
        real s = 0.0;
        for (int i = 0; i < n; i++) s += std::fabs(A(i, j));
        norm1 = std::max(norm1, s);
    }
    static const int degs[5] = { 3, 5, 7, 9, 13 };
    static const real theta[5] = { 1.495585217958292e-2,
                                   2.539398330063230e-1,
                                   9.504178996162932e-1,
                                   2.097847961257068e0,
                                   5.371920351148152e0 };
    int m = 13, s = 0;
    for (int k = 0; k < 4; k++)
        if (norm1 <= theta[k]) {
            m = degs[k];
            break;
        }
    rmat X = A;
    if (m == 13 && norm1 > theta[4]) {
        s = (int) std::ceil(std::log2(norm1 / theta[4]));
        X = scale(A, std::ldexp(1.0, -s));
    }
    /* Pade coefficients from the closed form */
    std::vector<long double> b(m + 1);
    for (int j = 0; j <= m; j++) {
        long double num = std::tgamma((long double) (2 * m - j + 1)) *
            std::tgamma((long double) (m + 1));
        long double den = std::tgamma((long double) (2 * m + 1)) *
            std::tgamma((long double) (j + 1)) *
            std::tgamma((long double) (m - j + 1));
        b[j] = num / den;
    }
    /* U = sum_{odd j} b_j X^j, V = sum_{even j} b_j X^j */
    rmat U(n, n), V(n, n), P = rmat::eye(n);
    for (int j = 0; j <= m; j++) {
        if (j > 0) P = mul(P, X);
        if (j % 2)
            U = add(U, P, (real) b[j]);
        else
            V = add(V, P, (real) b[j]);
    }
    rmat R = mul(inverse(add(V, U, -1.0)), add(V, U, 1.0));
    for (int k = 0; k < s; k++) R = mul(R, R);
    return R;
}

/* Cyclic Jacobi eigen-decomposition of a real symmetric matrix
 * (Golub & Van Loan sec. 8.5). Returns eigenvalues; columns of Q are the
 * eigenvectors. */
static std::vector<real> jacobi_sym(rmat A, rmat& Q)
{
    int n = A.n;
    Q = rmat::eye(n);
    for (int sweep = 0; sweep < 100; sweep++) {
        real off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                tot += A(i, j) * A(i, j);
                if (i != j) off += A(i, j) * A(i, j);
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                real apq = A(p, q);
                if (apq == 0.0) continue;
                real tau = (A(q, q) - A(p, p)) / (2.0 * apq);
                real t = (tau >= 0 ? 1.0 : -1.0) /
                    (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                real c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int k = 0; k < n; k++) {
                    real akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    real apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    real qkp = Q(k, p), qkq = Q(k, q);
                    Q(k, p) = c * qkp - s * qkq;
                    Q(k, q) = s * qkp + c * qkq;
                }
            }
    }
    std::vector<real> ev(n);
    for (int i = 0; i < n; i++) ev[i] = A(i, i);
    return ev;
}

/* Invariant planes of a real skew-symmetric U: vectors q1, q2 and
 * theta > 0 with U q1 = theta q2, U q2 = -theta q1, sorted by theta
 * descending (the order in which algo_lindblad_cvr_rodr.hpp:108-117 sorts
 * the Schur sub-diagonal). At most `kmax` planes. */
struct plane {
    real theta;
    std::vector<real> q1, q2;
};

static std::vector<plane> skew_planes(const rmat& U, int kmax)
{
    int n = U.n;
    rmat S = mul(transpose(U), U); /* = -U^2, symmetric PSD */
    rmat Q;
    std::vector<real> ev = jacobi_sym(S, Q);
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int i, int j) {
        return ev[i] > ev[j];
    });
    real evmax = n ? std::max(ev[order[0]], 0.0) : 0.0;
    std::vector<plane> planes;
    std::vector<std::vector<real> > basis;
    for (int idx : order) {
        if ((int) planes.size() >= kmax) break;
        if (!(ev[idx] > 1e-12 * evmax) || evmax == 0.0) break;
        std::vector<real> q(n);
        for (int i = 0; i < n; i++) q[i] = Q(i, idx);
        for (const auto& bv : basis) {
            real d = 0.0;
            for (int i = 0; i < n; i++) d += bv[i] * q[i];
            for (int i = 0; i < n; i++) q[i] -= d * bv[i];
        }
        real nq = 0.0;
        for (real v : q) nq += v * v;
        nq = std::sqrt(nq);
        if (nq < 0.1) continue; /* already spanned by a previous plane */
        for (real& v : q) v /= nq;
        std::vector<real> q2 = matvec(U, q);
        real th = 0.0;
        for (real v : q2) th += v * v;
        th = std::sqrt(th);
        if (th == 0.0) continue;
        for (real& v : q2) v /= th;
        basis.push_back(q);
        basis.push_back(q2);
        planes.push_back({ th, q, q2 });
    }
    return planes;
}

/* ------------------------------------------------------ qm description */

struct qm_desc {
    int N = 0;
    real carrier_density = 0.0;
    std::vector<real> h_diag, mu_diag;
    std::vector<cplx> h_off, mu_off;
    int relax_kind = MBG_RELAX_NONE;
    std::vector<std::vector<real> > scattering;
    std::vector<real> dephasing;
};

static qm_desc read_qm(const mbg_qm* q)
{
    qm_desc d;
    d.N = (int) q->num_levels;
    d.carrier_density = q->carrier_density;
    int no = d.N * (d.N - 1) / 2;
    d.h_diag.assign(q->h_diag, q->h_diag + d.N);
    d.mu_diag.assign(q->mu_diag, q->mu_diag + d.N);
    for (int i = 0; i < no; i++) {
        d.h_off.push_back(cplx(q->h_off[2 * i], q->h_off[2 * i + 1]));
        d.mu_off.push_back(cplx(q->mu_off[2 * i], q->mu_off[2 * i + 1]));
    }
    d.relax_kind = q->relax_kind;
    if (d.relax_kind == MBG_RELAX_LINDBLAD) {
        d.scattering.assign(d.N, std::vector<real>(d.N));
        for (int i = 0; i < d.N; i++)
            for (int j = 0; j < d.N; j++)
                d.scattering[i][j] = q->scattering[i * d.N + j];
        d.dephasing.assign(q->dephasing, q->dephasing + no);
    }
    return d;
}

/* qm_operator -> full matrix (coherence_vector_representation.hpp:99-130) */
static cmat op_to_mat(
    int N,
    const std::vector<real>& diag,
    const std::vector<cplx>& off)
{
    cmat m(N);
    for (int i = 0; i < N; i++) m(i, i) = diag[i];
    for (int i = 0, row = 0, col = 1; i < (int) off.size(); i++) {
        m(row, col) = off[i];
        m(col, row) = std::conj(off[i]);
        if (row == col - 1) {
            row = 0;
            col++;
        } else {
            row++;
        }
    }
    return m;
}

/* full matrix -> qm_operator parts (cvr.hpp:132-150) */
static void mat_to_op(
    const cmat& m,
    std::vector<real>& diag,
    std::vector<cplx>& off)
{
    int N = m.n;
    diag.assign(N, 0.0);
    off.clear();
    for (int i = 0; i < N; i++) diag[i] = m(i, i).real();
    for (int i = 1; i < N; i++)
        for (int j = 0; j < i; j++) off.push_back(m(j, i));
}

/* qm_lindblad_relaxation::action (qm_description.hpp:211-236); the base
 * qm_superop returns zeros (:127-132). */
static cmat relax_action(const qm_desc& q, const cmat& arg)
{
    int N = q.N;
    std::vector<real> diag;
    std::vector<cplx> off;
    mat_to_op(arg, diag, off);
    if (q.relax_kind != MBG_RELAX_LINDBLAD) {
        return cmat(N);
    }
    std::vector<real> pops(N, 0.0);
    for (int m = 0; m < N; m++) {
        real p = 0.0;
        for (int n = 0; n < N; n++) p += q.scattering[m][n] * diag[n];
        pops[m] = p;
    }
    for (size_t i = 0; i < off.size(); i++) off[i] *= q.dephasing[i];
    return op_to_mat(N, pops, off);
}

/* ------------------------------------------------ coherence vector repr. */

struct cvr {
    int N, V;
    std::vector<cmat> g;
    rmat ham, dip, relax;
    std::vector<real> dip_vec, equi;

    explicit cvr(const qm_desc& q) : N(q.N), V(q.N * q.N - 1)
    {
        /* generators u, v, w (cvr.hpp:52-93) */
        for (int k = 0; k < N; k++)
            for (int j = 0; j < k; j++) {
                cmat m(N);
                m(j, k) = 1;
                m(k, j) = 1;
                g.push_back(m);
            }
        for (int k = 0; k < N; k++)
            for (int j = 0; j < k; j++) {
                cmat m(N);
                m(j, k) = cplx(0, -1);
                m(k, j) = cplx(0, +1);
                g.push_back(m);
            }
        for (int l = 0; l < N - 1; l++) {
            cmat m(N);
            int j = 0;
            for (j = 0; j <= l; j++) m(j, j) = -1.0;
            m(j, j) = (real) (l + 1);
            int k = ((l + 1) * (l + 2)) / 2;
            for (auto& v : m.a) v /= std::sqrt((real) k);
            g.push_back(m);
        }
        cmat H = op_to_mat(N, q.h_diag, q.h_off);
        cmat mu = op_to_mat(N, q.mu_diag, q.mu_off);
        ham = liouvillian(H);
        dip = liouvillian(mu);
        dip_vec = op_vec(mu);
        /* relaxation superoperator (cvr.hpp:181-197) */
        relax = rmat(V, V);
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                cmat c = relax_action(q, g[j]);
                cmat d = cmul(c, g[i]);
                relax(i, j) = (0.5 * ctrace(d)).real();
            }
        /* equilibrium vector (cvr.hpp:199-213) */
        cmat I(N);
        for (int i = 0; i < N; i++) I(i, i) = 1.0;
        cmat d = relax_action(q, I);
        equi.assign(V, 0.0);
        for (int i = 0; i < V; i++) {
            cmat m = cmul(d, g[i]);
            real tr = 0.0;
            for (int k = 0; k < N; k++) tr += m(k, k).real();
            equi[i] = tr / N;
        }
    }

    /* cvr.hpp:149-166 */
    rmat liouvillian(const cmat& op) const
    {
        rmat r(V, V);
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                cmat gij = cmul(g[i], g[j]), gji = cmul(g[j], g[i]);
                cmat comm(N);
                for (size_t k = 0; k < comm.a.size(); k++)
                    comm.a[k] = gij.a[k] - gji.a[k];
                cmat res = cmul(op, comm);
                cplx c = cplx(0, 1) * 0.5 * ctrace(res);
                r(i, j) = c.real() * 1.0 / HBAR;
            }
        return r;
    }

    /* cvr.hpp:168-179 */
    std::vector<real> op_vec(const cmat& op) const
    {
        std::vector<real> r(V);
        for (int i = 0; i < V; i++) {
            cmat m = cmul(op, g[i]);
            real tr = 0.0;
            for (int k = 0; k < N; k++) tr += m(k, k).real();
            r[i] = tr;
        }
        return r;
    }
};

/* coherence vector of a density operator (cvr.hpp:341-394) */
static std::vector<real> coherence_vector(
    int N,
    const std::vector<real>& diag,
    const std::vector<cplx>& off)
{
    int V = N * N - 1;
    std::vector<real> r(V, 0.0);
    unsigned int i = 0;
    /* as in the reference, every off-diagonal entry writes index 0 of its
     * block; only the last entry's value survives (cvr.hpp:652-679) */
    for (size_t j = 0; j < off.size(); j++) r[i] = 2 * off[j].real();
    i = (N * (N - 1)) / 2;
    for (size_t j = 0; j < off.size(); j++) r[i] = -2 * off[j].imag();
    i = N * (N - 1);
    for (int l = 0; l < N - 1; l++) {
        int j = 0;
        real entry = 0;
        for (j = 0; j <= l; j++) entry += -1.0 * diag[j];
        entry += (l + 1) * diag[j];
        int k = ((l + 1) * (l + 2)) / 2;
        r[i + l] = entry / std::sqrt((real) k);
    }
    return r;
}

/* populations from a coherence vector (cvr.hpp:289-336) */
/* rho[row][col] (row != col) from the coherence vector: rho = I/N +
 * 1/2 sum_i d_i g_i with the generators of cvr.hpp:52-93 (u_jk: 1 at (j, k)
 * and (k, j); v_jk: -i at (j, k), +i at (k, j); pairs j < k in the order
 * k = 1..N-1, j = 0..k-1), so rho[j][k] = (d_u - i d_v) / 2 and
 * rho[k][j] its conjugate. No reference counterpart: the reference leaves
 * coherence records zero (solver_cpu_fdtd.tpp:314-318). */
static cplx cvr_coherence(int N, const real* d, unsigned int row, unsigned int col)
{
    unsigned int j = row < col ? row : col, k = row < col ? col : row;
    int P = N * (N - 1) / 2;
    int q = (int) (k * (k - 1) / 2 + j);
    cplx r(0.5 * d[q], -0.5 * d[P + q]);
    return row < col ? r : std::conj(r);
}

static real cvr_population(int N, const real* d, unsigned int m)
{
    if (N == 2) {
        return (m == 0) ? 0.5 - 0.5 * d[2] : 0.5 + 0.5 * d[2];
    } else if (N == 3) {
        switch (m) {
        case 0:
            return 1.0 / 3 + 0.5 * (-1.0 * d[6] - 1.0 / std::sqrt(3) * d[7]);
        case 1:
            return 1.0 / 3 + 0.5 * (+1.0 * d[6] - 1.0 / std::sqrt(3) * d[7]);
        case 2:
            return 1.0 / 3 + 0.5 * (+2.0 / std::sqrt(3) * d[7]);
        default:
            return 0.0;
        }
    }
    real sum = 0.0;
    for (int i = 0; i < N - 1; i++) {
        real factor;
        if ((int) m < i + 1)
            factor = -1.0;
        else if ((int) m == i + 1)
            factor = m;
        else
            factor = 0.0;
        int k = ((i + 1) * (i + 2)) / 2;
        sum += factor / std::sqrt((real) k) * d[N * (N - 1) + i];
    }
    return 1.0 / N + 0.5 * sum;
}

/* ------------------------------------------------ Lindblad: CVR/Rodrigues */

struct rodr_consts {
    bool has_qm = false;
    real M_CP = 0.0, d_t = 0.0, theta_1 = 0.0;
    rmat M, U, U2, A1;
    std::vector<rmat> coeff_1, coeff_2;
    std::vector<real> theta, v, d_eq, d_in;
};

/* algo_lindblad_cvr_rodr.hpp:143-229 */
static rodr_consts rodr_constants(const qm_desc* q, int N, real dt)
{
    rodr_consts sc;
    int V = N * N - 1;
    if (q) {
        if (q->N != N)
            throw std::invalid_argument(
                "Number of energy levels does not match selected solver!");
        sc.has_qm = true;
        cvr c(*q);
        sc.M_CP = 0.5 * q->carrier_density;
        sc.d_t = dt;
        sc.M = add(c.ham, c.relax);
        sc.U = scale(c.dip, -1.0);
        sc.U2 = mul(sc.U, sc.U);
        if (N == 2)
            sc.theta_1 = std::sqrt(
                std::pow(sc.U(0, 1), 2) + std::pow(sc.U(0, 2), 2) +
                std::pow(sc.U(1, 2), 2));
        sc.A1 = expm(scale(sc.M, dt / 2));
        /* fill_coefficients (rodr.hpp:101-136): planes of U */
        for (const auto& p : skew_planes(sc.U, V / 2)) {
            rmat c1(V, V), c2(V, V);
            for (int i = 0; i < V; i++)
                for (int j = 0; j < V; j++) {
                    c1(i, j) = p.q2[i] * p.q1[j] - p.q1[i] * p.q2[j];
                    c2(i, j) = -(p.q1[i] * p.q1[j] + p.q2[i] * p.q2[j]);
                }
            sc.coeff_1.push_back(c1);
            sc.coeff_2.push_back(c2);
            sc.theta.push_back(p.theta);
        }
        sc.v = c.dip_vec;
        sc.d_eq = c.equi;
        real eps = std::numeric_limits<real>::epsilon();
        bool zero = true;
        for (real x : sc.d_eq)
            if (std::fabs(x) > eps) zero = false;
        if (zero) {
            sc.d_in.assign(V, 0.0);
        } else {
            sc.d_in = solve_full_pivot(sc.M, sc.d_eq);
            std::vector<real> r = matvec(sc.M, sc.d_in);
            real nr = 0.0, nd = 0.0;
            for (int i = 0; i < V; i++) {
                nr += (r[i] - sc.d_eq[i]) * (r[i] - sc.d_eq[i]);
                nd += sc.d_eq[i] * sc.d_eq[i];
            }
            if (std::sqrt(nr) / std::sqrt(nd) > 1e-3)
                throw std::invalid_argument(
                    "Time-indepent matrix not invertible!");
        }
    } else {
        sc.has_qm = false;
        sc.M = rmat(V, V);
        sc.U = rmat(V, V);
        sc.U2 = rmat(V, V);
        sc.A1 = rmat(V, V);
        sc.v.assign(V, 0.0);
        sc.d_eq.assign(V, 0.0);
        sc.d_in.assign(V, 0.0);
    }
    return sc;
}

/* algo_lindblad_cvr_rodr.hpp:234-268. Inlined into callers with a constant
 * N (rodr_update_n), as the reference's update is instantiated per level
 * count; the arithmetic and its order are the same for every N. */
__attribute__((always_inline)) static inline void rodr_update(
    const rodr_consts& sc,
    int N,
    real* d,
    real e,
    real* p_t)
{
    if (!sc.has_qm) return;
    const int V = N * N - 1;
    real x[64], d1[64], d2[64];
    for (int i = 0; i < V; i++) x[i] = d[i] + sc.d_in[i];
    for (int i = 0; i < V; i++) {
        real s = 0.0;
        for (int j = 0; j < V; j++) s += sc.A1(i, j) * x[j];
        d1[i] = s - sc.d_in[i];
    }
    /* A2 (on the stack, like the reference's fixed-size matrices) */
    real A2[35 * 35];
    for (int i = 0; i < V * V; i++) A2[i] = 0.0;
    if (N == 2) {
        real th = sc.theta_1;
        real a = 0.0, b = 0.0;
        if (th != 0.0) {
            a = std::sin(th * e * sc.d_t) / th;
            b = (1 - std::cos(th * e * sc.d_t)) / (th * th);
        }
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++)
                A2[i * V + j] = a * sc.U(i, j) + b * sc.U2(i, j) +
                    (i == j ? 1.0 : 0.0);
    } else {
        for (int i = 0; i < V; i++) A2[i * V + i] = 1.0;
        for (size_t k = 0; k < sc.theta.size(); k++) {
            real s = std::sin(sc.theta[k] * e * sc.d_t);
            real c = 1 - std::cos(sc.theta[k] * e * sc.d_t);
            for (int i = 0; i < V * V; i++)
                A2[i] += s * sc.coeff_1[k].a[i] + c * sc.coeff_2[k].a[i];
        }
    }
    for (int i = 0; i < V; i++) {
        real s = 0.0;
        for (int j = 0; j < V; j++) s += A2[i * V + j] * d1[j];
        d2[i] = s + sc.d_in[i];
    }
    for (int i = 0; i < V; i++) {
        real s = 0.0;
        for (int j = 0; j < V; j++) s += sc.A1(i, j) * d2[j];
        d[i] = s - sc.d_in[i];
    }
    real acc = 0.0;
    for (int i = 0; i < V; i++) {
        real s = 0.0;
        for (int j = 0; j < V; j++) s += sc.M(i, j) * d[j];
        acc += sc.v[i] * (s + sc.d_eq[i]);
    }
    *p_t = sc.M_CP * acc;
}

template<int NL>
static void rodr_update_t(const rodr_consts& sc, real* d, real e, real* p_t)
{
    rodr_update(sc, NL, d, e, p_t);
}

static void rodr_update_n(const rodr_consts& sc, int N, real* d, real e, real* p_t)
{
    switch (N) {
    case 2: rodr_update_t<2>(sc, d, e, p_t); break;
    case 3: rodr_update_t<3>(sc, d, e, p_t); break;
    case 4: rodr_update_t<4>(sc, d, e, p_t); break;
    case 5: rodr_update_t<5>(sc, d, e, p_t); break;
    case 6: rodr_update_t<6>(sc, d, e, p_t); break;
    default: rodr_update(sc, N, d, e, p_t);
    }
}

/* --------------------------------------------------- Lindblad: Cayley */

struct cayley_consts {
    real dt = 0.0, carrier_dens = 0.0;
    cmat H0, mu;
    rmat d1, d2, D1, D2;
};

/* algo_lindblad_reg_cayley.hpp:123-203 */
static cayley_consts cayley_constants(const qm_desc* q, int N, real dt)
{
    cayley_consts sc;
    sc.dt = dt;
    sc.H0 = cmat(N);
    sc.mu = cmat(N);
    sc.d1 = rmat(N, N);
    sc.d2 = rmat(N, N);
    sc.D1 = rmat(N, N);
    sc.D2 = rmat(N, N);
    if (q) {
        if (q->N != N)
            throw std::invalid_argument(
                "Number of energy levels does not match selected solver!");
        sc.H0 = op_to_mat(N, q->h_diag, q->h_off);
        sc.mu = op_to_mat(N, q->mu_diag, q->mu_off);
        if (q->relax_kind != MBG_RELAX_LINDBLAD)
            throw std::invalid_argument("Unsupported superoperator!");
        for (int r = 0; r < N; r++)
            for (int c = 0; c < N; c++) sc.d1(r, c) = q->scattering[r][c];
        sc.D1 = expm(scale(sc.d1, dt / 2));
        for (int i = 0, row = 0, col = 1;
             row < N && col < N && i < (int) q->dephasing.size();
             i++) {
            sc.d2(row, col) = q->dephasing[i];
            sc.d2(col, row) = q->dephasing[i];
            if (row == col - 1) {
                row = 0;
                col++;
            } else {
                row++;
            }
        }
        for (int i = 0; i < N * N; i++)
            sc.D2.a[i] = std::exp(sc.d2.a[i] * dt / 2);
        sc.carrier_dens = q->carrier_density;
    }
    return sc;
}

/* propagate_dissipation (reg_cayley.hpp:206-217) */
static cmat cayley_dissipation(const cayley_consts& sc, const cmat& d)
{
    int N = d.n;
    cmat r(N);
    for (int i = 0; i < N * N; i++) r.a[i] = sc.D2.a[i] * d.a[i];
    for (int i = 0; i < N; i++) {
        cplx s(0, 0);
        for (int j = 0; j < N; j++) s += sc.D1(i, j) * d(j, j);
        r(i, i) = s;
    }
    return r;
}

/* reg_cayley.hpp:228-257 */
static void cayley_update(
    const cayley_consts& sc,
    cmat& d,
    real e,
    real* p_t)
{
    int N = d.n;
    cmat H(N);
    for (int i = 0; i < N * N; i++) H.a[i] = sc.H0.a[i] - e * sc.mu.a[i];
    cmat m(N);
    for (int i = 0; i < N * N; i++)
        m.a[i] = -cplx(0, 1) * 1.0 / HBAR * sc.dt * H.a[i];
    cmat Im(N), Ip(N);
    for (int i = 0; i < N; i++) {
        Im(i, i) = 1.0;
        Ip(i, i) = 1.0;
    }
    for (int i = 0; i < N * N; i++) {
        Im.a[i] -= 0.5 * m.a[i];
        Ip.a[i] += 0.5 * m.a[i];
    }
    cmat U2 = cmul(cinverse(Im), Ip);
    cmat d1 = cayley_dissipation(sc, d);
    cmat U2h(N);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) U2h(i, j) = std::conj(U2(j, i));
    cmat d2 = cmul(cmul(U2, d1), U2h);
    d = cayley_dissipation(sc, d2);
    cmat rhs_d(N);
    for (int i = 0; i < N * N; i++) rhs_d.a[i] = sc.d2.a[i] * d.a[i];
    for (int i = 0; i < N; i++) {
        cplx s(0, 0);
        for (int j = 0; j < N; j++) s += sc.d1(i, j) * d(j, j);
        rhs_d(i, i) = s;
    }
    cmat hd = cmul(sc.H0, d), dh = cmul(d, sc.H0);
    cmat rhs(N);
    for (int i = 0; i < N * N; i++)
        rhs.a[i] = -cplx(0, 1) * 1.0 / HBAR * (hd.a[i] - dh.a[i]) + rhs_d.a[i];
    *p_t = sc.carrier_dens * ctrace(cmul(rhs, sc.mu)).real();
}

/* ---------------------------------------------------------- the solver */

enum algo_t { ALGO_NOOP, ALGO_RODR, ALGO_CAYLEY };

struct record_plan {
    /* copy_list_entry_dev (copy_list_entry.hpp:51-109) */
    uint64_t offset_real = 0, offset_imag = 0, rows = 0, cols = 0,
             position_idx = 0;
    real interval_ratio = 1.0;
    int type = 0;
    uint32_t row_idx = 0, col_idx = 0;
    bool is_complex = false;
    bool coherence = false; /* record rho[row][col] (no reference
                               counterpart; the reference records zero) */

    bool hasto_record(uint64_t iteration) const
    {
        /* copy_list_entry.hpp:269-275; the reference evaluates
         * floor(ratio * (0 - 1)) on an unsigned wrap-around at iteration 0,
         * which never equals floor(0): iteration 0 always records. */
        if (iteration == 0) return true;
        long long last = (long long) std::floor(interval_ratio * (iteration - 1));
        long long next = (long long) std::floor(interval_ratio * (iteration + 0));
        return last != next;
    }
    int64_t offset(uint64_t iteration) const
    {
        return (int64_t) (offset_real +
                          std::floor(interval_ratio * iteration) * cols);
    }
};

struct solver {
    algo_t algo;
    int N;
    uint32_t n_x = 0, n_t = 0;
    real dx = 0, dt = 0, endtime = 0, dx_inv = 0;
    std::vector<real> e, h, p, fac_a, fac_b, fac_c, gamma;
    std::vector<uint32_t> mat_idx;
    int V = 0;
    std::vector<real> d_cvr;     /* n_x * V */
    std::vector<cmat> d_cay;     /* n_x */
    std::vector<rodr_consts> rodr;
    std::vector<cayley_consts> cay;
    std::vector<record_plan> records;
    std::vector<real> scratch;
    struct src {
        int type;
        uint32_t x_idx;
        std::vector<real> values;
    };
    std::vector<src> sources;
    uint64_t steps_done = 0;
    /* MBG_BC_MIRROR (no reference counterpart): H beyond the left end is
     * wall_l * E[0], beyond the right end -wall_r * E[n_x - 1]; 0 is the
     * reference's PMC boundary */
    real wall_l = 0, wall_r = 0;
};

/* common_fdtd.hpp:52-123 */
static void init_fdtd(
    const mbg_device* dev,
    const mbg_scenario* sc,
    real courant,
    uint32_t& n_x,
    uint32_t& n_t,
    real& dx,
    real& dt)
{
    if (sc->num_gridpoints == 0) throw std::invalid_argument("Invalid scenario.");
    real min_eps = 1e42, length = 0.0;
    for (uint32_t r = 0; r < dev->num_regions; r++) {
        const mbg_region& rg = dev->regions[r];
        real eps_r = dev->materials[rg.material].rel_permittivity;
        if (eps_r < min_eps) min_eps = eps_r;
        length += rg.x_end - rg.x_start;
    }
    real velocity = 1.0 / std::sqrt(MU0 * EPS0 * min_eps);
    n_x = sc->num_gridpoints;
    if (n_x == 1) {
        dx = 1e13;
        n_t = sc->num_timesteps;
        if (n_t < 2) throw std::invalid_argument("Invalid scenario.");
    } else {
        dx = length / (n_x - 1);
        real d_t = courant * dx / velocity;
        n_t = (unsigned int) (std::ceil(sc->endtime / d_t) + 1);
    }
    if (sc->endtime > std::numeric_limits<real>::min()) {
        dt = sc->endtime / (n_t - 1);
    } else {
        n_t = 1;
        dt = 3.154e10;
    }
}

static solver* create(
    const char* algo_name,
    uint32_t num_levels,
    const mbg_device* dev,
    const mbg_scenario* sc)
{
    std::unique_ptr<solver> s(new solver());
    std::string a(algo_name);
    if (a == "noop")
        s->algo = ALGO_NOOP;
    else if (a == "cvr-rodr")
        s->algo = ALGO_RODR;
    else if (a == "reg-cayley")
        s->algo = ALGO_CAYLEY;
    else
        throw std::invalid_argument("Unknown solver " + a);
    s->N = (int) num_levels;
    if (dev->num_regions == 0)
        throw std::invalid_argument("No regions in device!");
    init_fdtd(dev, sc, 0.5, s->n_x, s->n_t, s->dx, s->dt);
    s->endtime = sc->endtime;
    s->dx_inv = 1.0 / s->dx;
    uint32_t n = s->n_x;

    /* mirror walls: an impedance wall H = E / Z_w with
     * (Z_w - Z) / (Z_w + Z) = sqrt(refl), Z of the end point's material */
    if (dev->bc_kind == MBG_BC_MIRROR && n > 1) {
        auto wall = [&](real x, real refl) -> real {
            for (uint32_t r = 0; r < dev->num_regions; r++) {
                const mbg_region& rg = dev->regions[r];
                if (x >= rg.x_start && x <= rg.x_end) {
                    const mbg_material& mt = dev->materials[rg.material];
                    real z = std::sqrt(MU0 * mt.rel_permeability /
                                       (EPS0 * mt.rel_permittivity));
                    real zw = z * (1.0 + std::sqrt(refl)) / (1.0 - std::sqrt(refl));
                    return 1.0 / zw; /* 0 for refl = 1 */
                }
            }
            throw std::invalid_argument("region not found");
        };
        s->wall_l = wall(0.0, dev->refl_left);
        s->wall_r = wall((n - 1) * s->dx, dev->refl_right);
    }

    /* per-material constants (tpp:76-89): FDTD and Lindblad */
    struct fd {
        real a, b, c, g;
    };
    std::vector<fd> fdc;
    std::vector<qm_desc> qms(dev->num_materials);
    for (uint32_t m = 0; m < dev->num_materials; m++) {
        const mbg_material& mat = dev->materials[m];
        /* common_fdtd.hpp:158-190 */
        real sigma = std::sqrt(
                         EPS0 * mat.rel_permittivity /
                         (MU0 * mat.rel_permeability)) *
            mat.losses * 2.0;
        real epsilon = EPS0 * mat.rel_permittivity;
        real x = (sigma * s->dt) / (2.0 * epsilon);
        fd f;
        f.a = (1.0 - x) / (1.0 + x);
        f.b = s->dt / epsilon / (1.0 + x);
        f.c = s->dt / (MU0 * mat.rel_permeability * s->dx);
        f.g = mat.overlap_factor;
        fdc.push_back(f);
        const qm_desc* q = nullptr;
        if (mat.qm) {
            qms[m] = read_qm(mat.qm);
            q = &qms[m];
        }
        if (s->algo == ALGO_RODR)
            s->rodr.push_back(rodr_constants(q, s->N, s->dt));
        else if (s->algo == ALGO_CAYLEY)
            s->cay.push_back(cayley_constants(q, s->N, s->dt));
    }

    /* arrays and initial conditions (tpp:113-154) */
    s->e.assign(n, 0.0);
    s->h.assign(n + 1, 0.0);
    s->p.assign(n, 0.0);
    s->fac_a.assign(n, 0.0);
    s->fac_b.assign(n, 0.0);
    s->fac_c.assign(n, 0.0);
    s->gamma.assign(n, 0.0);
    s->mat_idx.assign(n, 0);
    if (s->algo == ALGO_RODR) {
        s->V = s->N * s->N - 1;
        s->d_cvr.assign((size_t) n * s->V, 0.0);
    } else if (s->algo == ALGO_CAYLEY) {
        s->d_cay.assign(n, cmat(s->N));
    }
    std::vector<real> rho_diag;
    std::vector<cplx> rho_off;
    if (sc->rho_levels) {
        rho_diag.assign(sc->rho_diag, sc->rho_diag + sc->rho_levels);
        for (uint32_t i = 0; i < sc->rho_num_off; i++)
            rho_off.push_back(cplx(sc->rho_off[2 * i], sc->rho_off[2 * i + 1]));
    }
    for (uint32_t i = 0; i < n; i++) {
        int idx = -1;
        bool has_qm = false;
        real x = i * s->dx;
        for (uint32_t r = 0; r < dev->num_regions; r++) {
            const mbg_region& rg = dev->regions[r];
            if ((x >= rg.x_start) && (x <= rg.x_end)) {
                idx = (int) rg.material;
                has_qm = dev->materials[rg.material].qm != nullptr;
                break;
            }
        }
        if ((idx < 0) || (idx >= (int) dev->num_materials))
            throw std::invalid_argument("region not found");
        s->fac_a[i] = fdc[idx].a;
        s->fac_b[i] = fdc[idx].b;
        s->fac_c[i] = fdc[idx].c;
        s->gamma[i] = fdc[idx].g;
        s->mat_idx[i] = (uint32_t) idx;
        if (has_qm) {
            if (s->algo == ALGO_RODR) {
                std::vector<real> d =
                    coherence_vector(s->N, rho_diag, rho_off);
                std::copy(d.begin(), d.end(), &s->d_cvr[(size_t) i * s->V]);
            } else if (s->algo == ALGO_CAYLEY) {
                cmat m(s->N);
                for (int k = 0; k < s->N; k++) m(k, k) = rho_diag[k];
                for (int k = 0, row = 0, col = 1;
                     row < s->N && col < s->N && k < (int) rho_off.size();
                     k++) {
                    m(row, col) = rho_off[k];
                    m(col, row) = std::conj(rho_off[k]);
                    if (row == col - 1) {
                        row = 0;
                        col++;
                    } else {
                        row++;
                    }
                }
                s->d_cay[i] = m;
            }
        }
        s->e[i] = (sc->e_init_kind == MBG_FIELD_IC_VALUES)
            ? sc->e_init_values[i]
            : sc->e_init_value;
        s->h[i] = (sc->h_init_kind == MBG_FIELD_IC_VALUES)
            ? sc->h_init_values[i]
            : sc->h_init_value;
    }
    s->h[n] = 0.0;

    /* record plan (tpp:157-182, copy_list_entry.hpp:127-171) */
    uint64_t scratch_size = 0;
    for (uint32_t k = 0; k < sc->num_records; k++) {
        const mbg_record& rec = sc->records[k];
        record_plan rp;
        if (rec.interval <= s->dt) {
            rp.rows = s->n_t;
            rp.interval_ratio = 1.0;
        } else {
            rp.rows = (uint64_t) (std::floor(s->endtime / rec.interval) + 1);
            rp.interval_ratio = s->dt / rec.interval;
        }
        if (rec.position < 0.0) {
            rp.position_idx = 0;
            rp.cols = n;
        } else {
            rp.position_idx = (uint64_t) std::round(rec.position / s->dx);
            rp.cols = 1;
        }
        rp.type = rec.type;
        rp.is_complex = rec.is_complex != 0;
        rp.row_idx = rec.row;
        rp.col_idx = rec.col;
        rp.coherence = rec.coherence != 0 && rec.row != rec.col &&
            rec.type == MBG_RECORD_DENSITY;
        rp.offset_real = scratch_size;
        rp.offset_imag = scratch_size + rp.cols * rp.rows;
        scratch_size += rp.cols * rp.rows;
        if (rp.is_complex) scratch_size += rp.cols * rp.rows;
        s->records.push_back(rp);
    }
    s->scratch.assign(scratch_size, 0.0);

    /* sources (tpp:185-202, source.hpp:94-106) */
    for (uint32_t k = 0; k < sc->num_sources; k++) {
        const mbg_source& src = sc->sources[k];
        solver::src ss;
        ss.type = src.type;
        ss.x_idx = (unsigned int) (src.position / s->dx);
        ss.values.resize(s->n_t);
        for (uint32_t j = 0; j < s->n_t; j++) {
            real t = j * s->dt;
            real v = 0.0;
            if (src.shape == MBG_SHAPE_SECH) {
                v = src.ampl *
                    (1 / std::cosh(src.beta_or_tau * t - src.phase) *
                     std::sin(2 * PI * src.freq * t - src.phase_sin));
            } else if (src.shape == MBG_SHAPE_GAUSSIAN) {
                real tau = src.beta_or_tau;
                v = src.ampl *
                    (std::exp(-(t - src.phase) * (t - src.phase) / (tau * tau)) *
                     std::sin(2 * PI * src.freq * t));
            } else {
                if (j >= src.table_len)
                    throw std::invalid_argument("source table too short");
                v = src.table[j];
            }
            ss.values[j] = v;
        }
        s->sources.push_back(ss);
    }
    return s.release();
}

/* rho[row][col] of a coherence record at point i (see cvr_coherence) */
/* The state a record reads: the solver's arrays, or a thread's private
 * copy of a range of them (grid point i at index i - base). */
struct view {
    const real* e;
    const real* h;
    const real* p;
    const real* d_cvr;
    const cmat* d_cay;
    int64_t base;
};

static view full_view(const solver* s)
{
    return view{ s->e.data(), s->h.data(), s->p.data(), s->d_cvr.data(), s->d_cay.data(), 0 };
}

/* rho[row][col] of a coherence record at point i (see cvr_coherence) */
static cplx coherence_value(const solver* s, const view& w, const record_plan& rp, uint64_t i)
{
    const int64_t k = (int64_t) i - w.base;
    if (s->algo == ALGO_RODR)
        return cvr_coherence(s->N, &w.d_cvr[k * s->V], rp.row_idx, rp.col_idx);
    if (s->algo == ALGO_CAYLEY) return w.d_cay[k](rp.row_idx, rp.col_idx);
    return cplx(0.0, 0.0);
}

static real record_value(const solver* s, const view& w, const record_plan& rp, uint64_t i)
{
    if (rp.coherence) return coherence_value(s, w, rp, i).real();
    const int64_t k = (int64_t) i - w.base;
    switch (rp.type) {
    case MBG_RECORD_ELECTRIC:
        return w.e[k];
    case MBG_RECORD_POLAR_DT:
        return w.p[k];
    case MBG_RECORD_MAGNETIC:
        return w.h[k];
    case MBG_RECORD_INVERSION:
        if (s->algo == ALGO_RODR)
            return w.d_cvr[k * s->V + s->N * (s->N - 1)];
        if (s->algo == ALGO_CAYLEY)
            return (w.d_cay[k](1, 1) - w.d_cay[k](0, 0)).real();
        return 0.0;
    case MBG_RECORD_DENSITY:
        if (rp.row_idx != rp.col_idx) return 0.0; /* coherences: TODO in ref */
        if (s->algo == ALGO_RODR)
            return cvr_population(s->N, &w.d_cvr[k * s->V], rp.row_idx);
        if (s->algo == ALGO_CAYLEY)
            return w.d_cay[k](rp.row_idx, rp.row_idx).real();
        return 0.0;
    default:
        return 0.0;
    }
}

/* solver_cpu_fdtd::run (tpp:223-338); max_steps bounds a timing sample */
static void run(solver* s, int threads, uint32_t max_steps)
{
    const int64_t n = s->n_x;
    uint32_t steps = s->n_t;
    if (max_steps && max_steps < steps) steps = max_steps;
    real* E = s->e.data();
    real* H = s->h.data();
    real* P = s->p.data();
    const real* fa = s->fac_a.data();
    const real* fb = s->fac_b.data();
    const real* fc = s->fac_c.data();
    const real* ga = s->gamma.data();
    const uint32_t* mi = s->mat_idx.data();
    const real dxi = s->dx_inv;
    if (threads < 1) threads = 1;
#pragma omp parallel num_threads(threads)
    {
        for (uint32_t t = 0; t < steps; t++) {
            // USE_OMP_SIMD (the CPU-baseline build): the reference's
            // vectorised field loops (solver_cpu_fdtd.tpp:233-236, 258-261)
#if USE_OMP_SIMD
#pragma omp for simd schedule(static)
#else
#pragma omp for schedule(static)
#endif
            for (int64_t i = 0; i < n; i++)
                E[i] = fa[i] * E[i] +
                    fb[i] * (-ga[i] * P[i] + (H[i + 1] - H[i]) * dxi);
#pragma omp single
            for (const auto& src : s->sources) {
                if (src.type == MBG_SOURCE_HARD)
                    E[src.x_idx] = src.values[t];
                else if (src.type == MBG_SOURCE_SOFT)
                    E[src.x_idx] += src.values[t];
            }
#if USE_OMP_SIMD
#pragma omp for simd schedule(static)
#else
#pragma omp for schedule(static)
#endif
            for (int64_t i = 1; i < n; i++) H[i] += fc[i] * (E[i] - E[i - 1]);
#pragma omp single
            {
                H[0] = s->wall_l != 0 ? s->wall_l * E[0] : 0;
                H[n] = s->wall_r != 0 ? -s->wall_r * E[n - 1] : 0;
            }
            if (s->algo == ALGO_RODR) {
#pragma omp for schedule(static)
                for (int64_t i = 0; i < n; i++)
                    rodr_update_n(
                        s->rodr[mi[i]], s->N, &s->d_cvr[i * s->V], E[i], &P[i]);
            } else if (s->algo == ALGO_CAYLEY) {
#pragma omp for schedule(static)
                for (int64_t i = 0; i < n; i++)
                    cayley_update(s->cay[mi[i]], s->d_cay[i], E[i], &P[i]);
            }
            for (const auto& rp : s->records) {
                if (!rp.hasto_record(t)) continue;
                uint64_t pos = rp.position_idx, cols = rp.cols;
                int64_t o_r = rp.offset(t);
                if ((uint64_t) (o_r - (int64_t) rp.offset_real) >= rp.rows * cols)
                    continue; /* row outside the result (guard) */
                const view w = full_view(s);
#pragma omp for schedule(static)
                for (int64_t i = (int64_t) pos; i < (int64_t) (pos + cols); i++)
                    if (i < n) s->scratch[o_r + i - pos] = record_value(s, w, rp, i);
                if (rp.coherence) {
                    int64_t o_i = o_r - (int64_t) rp.offset_real + (int64_t) rp.offset_imag;
#pragma omp for schedule(static)
                    for (int64_t i = (int64_t) pos; i < (int64_t) (pos + cols); i++)
                        if (i < n) s->scratch[o_i + i - pos] = coherence_value(s, w, rp, i).imag();
                }
            }
        }
    }
    s->steps_done += steps;
}

/* solver_cpu_fdtd_red::run (red.tpp:351-567) restated: each thread owns a
 * contiguous range of points and, every `ol` steps, copies that range
 * widened by ol points on each side into private arrays, advances the
 * copy by up to ol steps, and writes its own range back. Garbage enters a
 * copy from its open edges by one point per step, so the owned range stays
 * exact; the arithmetic of every point and step is that of run() (same
 * order: E, sources, H and boundary, density, records), so the results
 * equal run()'s bit for bit. Two barriers per ol steps instead of several
 * per step: the loop for small runs on many cores. Falls back to run()
 * when a thread would own fewer than 2 ol points. */
static void run_red(solver* s, int threads, uint32_t max_steps, int ol)
{
    const int64_t n = s->n_x;
    uint32_t steps = s->n_t;
    if (max_steps && max_steps < steps) steps = max_steps;
    if (threads < 1) threads = 1;
    if (ol < 1) ol = 1;
    if (n < (int64_t) threads * 2 * ol) {
        run(s, threads, max_steps);
        return;
    }
    const int V = s->V;
    const real dxi = s->dx_inv;
#pragma omp parallel num_threads(threads)
    {
        const int t = omp_get_thread_num();
        const int nt = omp_get_num_threads();
        const int64_t chunk = n / nt;
        const int64_t b = t * chunk, e = (t == nt - 1) ? n : b + chunk;
        const int64_t lo = std::max<int64_t>(0, b - ol), hi = std::min<int64_t>(n, e + ol);
        const int64_t m = hi - lo;
        std::vector<real> E(m), H(m + 1), P(m), D(s->algo == ALGO_RODR ? (size_t) m * V : 0);
        std::vector<cmat> R(s->algo == ALGO_CAYLEY ? m : 0);
        const view w{ E.data(), H.data(), P.data(), D.data(), R.data(), lo };
        for (uint32_t t0 = 0; t0 < steps; t0 += (uint32_t) ol) {
            const uint32_t nsub = std::min<uint32_t>((uint32_t) ol, steps - t0);
            std::copy(s->e.begin() + lo, s->e.begin() + hi, E.begin());
            std::copy(s->h.begin() + lo, s->h.begin() + hi + 1, H.begin());
            std::copy(s->p.begin() + lo, s->p.begin() + hi, P.begin());
            if (s->algo == ALGO_RODR)
                std::copy(s->d_cvr.begin() + lo * V, s->d_cvr.begin() + hi * V, D.begin());
            else if (s->algo == ALGO_CAYLEY)
                std::copy(s->d_cay.begin() + lo, s->d_cay.begin() + hi, R.begin());
#pragma omp barrier
            // local pointers shifted to the copy's first point, as run()'s
            // plain arrays (so that the loops vectorise alike)
            real* __restrict__ Ep = E.data();
            real* __restrict__ Hp = H.data();
            real* __restrict__ Pp = P.data();
            const real* __restrict__ fa = s->fac_a.data() + lo;
            const real* __restrict__ fb = s->fac_b.data() + lo;
            const real* __restrict__ fc = s->fac_c.data() + lo;
            const real* __restrict__ ga = s->gamma.data() + lo;
            const uint32_t* mi = s->mat_idx.data() + lo;
            for (uint32_t k = 0; k < nsub; k++) {
                const uint32_t step = t0 + k;
                // (red.tpp:300-301, 318-319 under USE_OMP_SIMD)
#if USE_OMP_SIMD
#pragma omp simd
#endif
                for (int64_t i = 0; i < m; i++)
                    Ep[i] = fa[i] * Ep[i] + fb[i] * (-ga[i] * Pp[i] + (Hp[i + 1] - Hp[i]) * dxi);
                for (const auto& src : s->sources) {
                    const int64_t x = src.x_idx;
                    if (x < lo || x >= hi) continue;
                    if (src.type == MBG_SOURCE_HARD)
                        Ep[x - lo] = src.values[step];
                    else if (src.type == MBG_SOURCE_SOFT)
                        Ep[x - lo] += src.values[step];
                }
#if USE_OMP_SIMD
#pragma omp simd
#endif
                for (int64_t i = 1; i < m; i++) Hp[i] += fc[i] * (Ep[i] - Ep[i - 1]);
                if (lo == 0) Hp[0] = s->wall_l != 0 ? s->wall_l * Ep[0] : 0;
                if (hi == n) Hp[m] = s->wall_r != 0 ? -s->wall_r * Ep[m - 1] : 0;
                if (s->algo == ALGO_RODR) {
                    for (int64_t i = 0; i < m; i++)
                        rodr_update_n(s->rodr[mi[i]], s->N, &D[i * V], Ep[i], &Pp[i]);
                } else if (s->algo == ALGO_CAYLEY) {
                    for (int64_t i = 0; i < m; i++)
                        cayley_update(s->cay[mi[i]], R[i], Ep[i], &Pp[i]);
                }
                for (const auto& rp : s->records) {
                    if (!rp.hasto_record(step)) continue;
                    const int64_t pos = (int64_t) rp.position_idx, cols = (int64_t) rp.cols;
                    const int64_t o_r = rp.offset(step);
                    if ((uint64_t) (o_r - (int64_t) rp.offset_real) >= rp.rows * rp.cols) continue;
                    const int64_t r0 = std::max(pos, b), r1 = std::min(pos + cols, e);
                    for (int64_t i = r0; i < r1; i++) {
                        s->scratch[o_r + i - pos] = record_value(s, w, rp, i);
                        if (rp.coherence)
                            s->scratch[o_r - (int64_t) rp.offset_real + (int64_t) rp.offset_imag + i - pos] =
                                coherence_value(s, w, rp, i).imag();
                    }
                }
            }
            // the owned range back; H at the owned points (and H[n] for the
            // last range)
            std::copy(E.begin() + (b - lo), E.begin() + (e - lo), s->e.begin() + b);
            std::copy(H.begin() + (b - lo), H.begin() + (e - lo) + (e == n ? 1 : 0), s->h.begin() + b);
            std::copy(P.begin() + (b - lo), P.begin() + (e - lo), s->p.begin() + b);
            if (s->algo == ALGO_RODR)
                std::copy(D.begin() + (b - lo) * V, D.begin() + (e - lo) * V, s->d_cvr.begin() + b * V);
            else if (s->algo == ALGO_CAYLEY)
                std::copy(R.begin() + (b - lo), R.begin() + (e - lo), s->d_cay.begin() + b);
#pragma omp barrier
        }
    }
    s->steps_done += steps;
}

} // namespace mbo

/* ------------------------------------------------------------- C-ABI */

static thread_local std::string g_err;

template<typename F>
static int guard(F f)
{
    try {
        f();
        return MBG_OK;
    } catch (const std::invalid_argument& e) {
        g_err = e.what();
        return MBG_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        g_err = e.what();
        return MBG_ERR_RUNTIME;
    }
}

extern "C" {

typedef struct mbo_solver mbo_solver;

const char* mbo_last_error(void) { return g_err.c_str(); }

int mbo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int mbo_create(
    const char* algo,
    uint32_t num_levels,
    const mbg_device* dev,
    const mbg_scenario* scen,
    mbo_solver** out)
{
    return guard([&] {
        *out = (mbo_solver*) mbo::create(algo, num_levels, dev, scen);
    });
}

int mbo_grid(const mbo_solver* h, mbg_grid* g)
{
    const mbo::solver* s = (const mbo::solver*) h;
    g->num_gridpoints = s->n_x;
    g->num_timesteps = s->n_t;
    g->gridpoint_size = s->dx;
    g->timestep_size = s->dt;
    g->endtime = s->endtime;
    return MBG_OK;
}

int mbo_run(mbo_solver* h, int threads, uint32_t max_steps)
{
    return guard([&] { mbo::run((mbo::solver*) h, threads, max_steps); });
}

/* the temporally blocked loop (solver_cpu_fdtd_red), overlap `ol` steps */
int mbo_run_red(mbo_solver* h, int threads, uint32_t max_steps, int ol)
{
    return guard([&] { mbo::run_red((mbo::solver*) h, threads, max_steps, ol); });
}

int mbo_num_results(const mbo_solver* h, uint32_t* n)
{
    *n = (uint32_t) ((const mbo::solver*) h)->records.size();
    return MBG_OK;
}

int mbo_result_shape(
    const mbo_solver* h,
    uint32_t k,
    uint32_t* rows,
    uint32_t* cols,
    int32_t* is_complex)
{
    const mbo::solver* s = (const mbo::solver*) h;
    if (k >= s->records.size()) {
        g_err = "result index out of range";
        return MBG_ERR_INVALID_ARGUMENT;
    }
    *rows = (uint32_t) s->records[k].rows;
    *cols = (uint32_t) s->records[k].cols;
    *is_complex = s->records[k].is_complex;
    return MBG_OK;
}

int mbo_copy_result(const mbo_solver* h, uint32_t k, double* re, double* im)
{
    const mbo::solver* s = (const mbo::solver*) h;
    if (k >= s->records.size()) {
        g_err = "result index out of range";
        return MBG_ERR_INVALID_ARGUMENT;
    }
    const auto& rp = s->records[k];
    uint64_t size = rp.rows * rp.cols;
    std::copy(
        s->scratch.begin() + rp.offset_real,
        s->scratch.begin() + rp.offset_real + size,
        re);
    if (im && rp.is_complex)
        std::copy(
            s->scratch.begin() + rp.offset_imag,
            s->scratch.begin() + rp.offset_imag + size,
            im);
    return MBG_OK;
}

/* State snapshot: E[n], H[n+1], P[n] and the density (V or 2N^2 reals per
 * point: CVR vector, or Cayley (re, im) row-major). */
int mbo_state(
    const mbo_solver* h,
    double* e,
    double* hh,
    double* p,
    double* d)
{
    const mbo::solver* s = (const mbo::solver*) h;
    if (e) std::copy(s->e.begin(), s->e.end(), e);
    if (hh) std::copy(s->h.begin(), s->h.end(), hh);
    if (p) std::copy(s->p.begin(), s->p.end(), p);
    if (d) {
        if (s->algo == mbo::ALGO_RODR)
            std::copy(s->d_cvr.begin(), s->d_cvr.end(), d);
        else if (s->algo == mbo::ALGO_CAYLEY) {
            size_t o = 0;
            for (const auto& m : s->d_cay)
                for (const auto& v : m.a) {
                    d[o++] = v.real();
                    d[o++] = v.imag();
                }
        }
    }
    return MBG_OK;
}

/* Rodrigues constants of one material for unit tests: M, U, A1 (V x V
 * each), theta[V/2] (zero-padded), v, d_eq, d_in (V each), M_CP; the
 * matrix exp(s U) assembled from the planes for s = probe (V x V). */
int mbo_rodr_constants(
    const mbg_qm* q,
    double dt,
    double probe,
    double* M,
    double* U,
    double* A1,
    double* theta,
    double* v,
    double* d_eq,
    double* d_in,
    double* m_cp,
    double* A2_probe)
{
    return guard([&] {
        mbo::qm_desc d = mbo::read_qm(q);
        mbo::rodr_consts c = mbo::rodr_constants(&d, d.N, dt);
        int V = d.N * d.N - 1;
        std::copy(c.M.a.begin(), c.M.a.end(), M);
        std::copy(c.U.a.begin(), c.U.a.end(), U);
        std::copy(c.A1.a.begin(), c.A1.a.end(), A1);
        for (int k = 0; k < V / 2; k++)
            theta[k] = k < (int) c.theta.size() ? c.theta[k] : 0.0;
        std::copy(c.v.begin(), c.v.end(), v);
        std::copy(c.d_eq.begin(), c.d_eq.end(), d_eq);
        std::copy(c.d_in.begin(), c.d_in.end(), d_in);
        *m_cp = c.M_CP;
        for (int i = 0; i < V * V; i++) A2_probe[i] = (i % (V + 1) == 0);
        for (size_t k = 0; k < c.theta.size(); k++) {
            double s = std::sin(c.theta[k] * probe);
            double cc = 1 - std::cos(c.theta[k] * probe);
            for (int i = 0; i < V * V; i++)
                A2_probe[i] += s * c.coeff_1[k].a[i] + cc * c.coeff_2[k].a[i];
        }
    });
}

/* Matrix exponential of a real n x n row-major matrix (unit tests). */
int mbo_expm(int n, const double* a, double* out)
{
    return guard([&] {
        mbo::rmat A(n, n);
        std::copy(a, a + n * n, A.a.begin());
        mbo::rmat R = mbo::expm(A);
        std::copy(R.a.begin(), R.a.end(), out);
    });
}

void mbo_destroy(mbo_solver* h) { delete (mbo::solver*) h; }

} /* extern "C" */
