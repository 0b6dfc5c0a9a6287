// CPU oracle for the DiffStir MLS-MPM stirring path.
//
// TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline / reference arm may load this library, and only as the
// checker or the timed CPU stand-in for the reference; the product path
// (diffstir_gb300) never calls it.
//
// It restates, line by line and in scalar code templated on the float type,
// the reference's Taichi kernels in src/simulator/simulation_functions.py:
//   compute_F_tmp :39-42, p2g :104-196, grid_op :199-225, g2p :228-290,
//   compute_loss :330-339, backward_svd/clamp :61-87,
// with the constants of src/simulator/initialization.py:14-54 carried in
// DstirSceneDesc (include/diffstir.h).  Two additions that the reference does
// not have are switchable and off in the reference scene: the analytic moving
// cylinder rod (DSTIR_ROD_CYLINDER) and J taken from the SVD (DSTIR_J_SVD).
//
// The reverse pass is a hand-derived adjoint of exactly these equations
// (Taichi's autodiff generated the reference's .grad kernels); it takes the
// same branches as the forward pass, abs -> sign, and d||C||/dC = 0 at C = 0.
// Parity of this restatement is pinned by tests/golden (fixtures produced by
// executing the reference's own source through a Taichi-semantics shim) and by
// central finite differences of the FP64 build.
//
// With threads > 1 the scatters use thread-private grids summed in a fixed
// order, so results are deterministic for a given thread count.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/diffstir.h"

namespace {

#ifdef ORACLE_BRANCH_COUNTS
// Diagnostic build: how often each boundary rule of grid_op (:204-224)
// changed the velocity of a node with mass, summed over the forward substeps
// of every rollout since the last oracle_branch_counts call.  Index:
// 0 container projection, 1 wall i<b, 2 wall i>n-b, 3 wall k<b, 4 wall k>n-b,
// 5 wall j<b, 6 sticky top, 7 nodes with mass visited.
constexpr int NBRANCH = 8;
long long g_branch[NBRANCH];
inline void count_branch(int b) {
#pragma omp atomic
    g_branch[b]++;
}
#define BRANCH(b) count_branch(b)
#else
#define BRANCH(b) ((void)0)
#endif

constexpr int NS = 24;  // per-particle state: x3 v3 C9 F9
constexpr int OX = 0, OV = 3, OC = 6, OF = 15;

template <class R>
struct Mat3 {
    R a[9];
};

template <class R>
inline void matmul(const R* A, const R* B, R* out) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R s = A[i * 3 + 0] * B[0 * 3 + j];
            s += A[i * 3 + 1] * B[1 * 3 + j];
            s += A[i * 3 + 2] * B[2 * 3 + j];
            out[i * 3 + j] = s;
        }
}

template <class R>
inline R det3(const R* a) {
    // same cofactor expansion along row 0 as Taichi's Matrix.determinant
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

template <class R>
inline void cof3(const R* a, R* c) {
    // d det / d a
    c[0] = a[4] * a[8] - a[5] * a[7];
    c[1] = -(a[3] * a[8] - a[5] * a[6]);
    c[2] = a[3] * a[7] - a[4] * a[6];
    c[3] = -(a[1] * a[8] - a[2] * a[7]);
    c[4] = a[0] * a[8] - a[2] * a[6];
    c[5] = -(a[0] * a[7] - a[1] * a[6]);
    c[6] = a[1] * a[5] - a[2] * a[4];
    c[7] = -(a[0] * a[5] - a[2] * a[3]);
    c[8] = a[0] * a[4] - a[1] * a[3];
}

// quadratic B-spline weights and derivatives, simulation_functions.py:108-110
template <class R>
inline void bspline(const R fx[3], R w[3][3], R dw[3][3]) {
    for (int d = 0; d < 3; ++d) {
        R t0 = R(1.5) - fx[d], t1 = fx[d] - R(1), t2 = fx[d] - R(0.5);
        w[0][d] = R(0.5) * t0 * t0;
        w[1][d] = R(0.75) - t1 * t1;
        w[2][d] = R(0.5) * t2 * t2;
        dw[0][d] = -t0;
        dw[1][d] = R(-2) * t1;
        dw[2][d] = t2;
    }
}

// Viscosity and its partials, simulation_functions.py:118-146.
template <class R>
struct Visc {
    R eta;
    R deta_dgamma;
    R deta_dp[4];
};

template <class R>
inline Visc<R> viscosity(int model, const R* prm, R gamma) {
    Visc<R> o{};
    if (model == DSTIR_MODEL_CARREAU) {
        R eta0 = prm[0], einf = prm[1], n = prm[2], lam = prm[3];
        R lg = lam * gamma;
        R B = R(1) + lg * lg;
        R e = (n - R(1)) / R(2);
        R Be = std::pow(B, e);
        o.eta = einf + (eta0 - einf) * Be;
        R dBe_dB = e * std::pow(B, e - R(1));
        o.deta_dp[0] = Be;
        o.deta_dp[1] = R(1) - Be;
        o.deta_dp[2] = (eta0 - einf) * Be * std::log(B) * R(0.5);
        o.deta_dp[3] = (eta0 - einf) * dBe_dB * R(2) * lg * gamma;
        o.deta_dp[3] = o.deta_dp[3];
        o.deta_dgamma = (eta0 - einf) * dBe_dB * R(2) * lg * lam;
    } else if (model == DSTIR_MODEL_CROSS) {
        R eta0 = prm[0], einf = prm[1], n = prm[2], lam = prm[3];
        R lg = lam * gamma;
        R q = std::pow(lg, n - R(1));
        R inv = R(1) / (R(1) + q);
        o.eta = einf + (eta0 - einf) * inv;
        R deta_dq = -(eta0 - einf) * inv * inv;
        R dq_dlg = (n - R(1)) * std::pow(lg, n - R(2));
        o.deta_dp[0] = inv;
        o.deta_dp[1] = R(1) - inv;
        o.deta_dp[2] = deta_dq * q * std::log(lg);
        o.deta_dp[3] = deta_dq * dq_dlg * gamma;
        o.deta_dgamma = deta_dq * dq_dlg * lam;
    } else {  // Herschel-Bulkley
        R K = prm[0], tau = prm[1], n = prm[2];
        R gp = std::pow(gamma, n - R(1));
        R delta = K * gp;
        o.eta = tau / gamma;
        o.deta_dgamma = -tau / (gamma * gamma);
        o.deta_dp[1] = R(1) / gamma;
        if (delta > R(0)) {
            o.eta += delta;
            o.deta_dp[0] = gp;
            o.deta_dp[2] = delta * std::log(gamma);
            o.deta_dgamma += K * (n - R(1)) * std::pow(gamma, n - R(2));
        }
    }
    return o;
}

// ---------------------------------------------------------------------------
// 3x3 SVD (one-sided Jacobi on A^T A, then Givens QR of A V), double only.
// Convention of the reference's ti.svd: det U = det V = +1, the smallest
// singular value carries the sign of det A, values sorted by magnitude.
// ---------------------------------------------------------------------------
inline void jacobi_eig3(double S[9], double V[9]) {
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = S[1] * S[1] + S[2] * S[2] + S[5] * S[5];
        double diag = S[0] * S[0] + S[4] * S[4] + S[8] * S[8];
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int pq = 0; pq < 3; ++pq) {
            int p = (pq == 2) ? 1 : 0, q = (pq == 0) ? 1 : 2;
            double apq = S[p * 3 + q];
            if (apq == 0.0) continue;
            double app = S[p * 3 + p], aqq = S[q * 3 + q];
            double theta = (aqq - app) / (2.0 * apq);
            double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
            double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
            // S <- G^T S G with G = rotation in (p,q)
            for (int k = 0; k < 3; ++k) {
                double skp = S[k * 3 + p], skq = S[k * 3 + q];
                S[k * 3 + p] = c * skp - s * skq;
                S[k * 3 + q] = s * skp + c * skq;
            }
            for (int k = 0; k < 3; ++k) {
                double spk = S[p * 3 + k], sqk = S[q * 3 + k];
                S[p * 3 + k] = c * spk - s * sqk;
                S[q * 3 + k] = s * spk + c * sqk;
            }
            for (int k = 0; k < 3; ++k) {
                double vkp = V[k * 3 + p], vkq = V[k * 3 + q];
                V[k * 3 + p] = c * vkp - s * vkq;
                V[k * 3 + q] = s * vkp + c * vkq;
            }
        }
    }
}

inline void svd3_d(const double A[9], double U[9], double sig[3], double V[9]) {
    double S[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += A[k * 3 + i] * A[k * 3 + j];
            S[i * 3 + j] = s;
        }
    jacobi_eig3(S, V);
    double ev[3] = {S[0], S[4], S[8]};
    // sort eigenvalues descending, permuting columns of V
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int a, int b) { return ev[a] > ev[b]; });
    double Vs[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Vs[r * 3 + c] = V[r * 3 + ord[c]];
    double detV = det3(Vs);
    if (detV < 0)
        for (int r = 0; r < 3; ++r) Vs[r * 3 + 2] = -Vs[r * 3 + 2];
    // B = A V, then QR by Givens rotations: B = U R
    double B[9];
    matmul(A, Vs, B);
    double Q[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    auto givens = [&](int r1, int r2, int col) {
        double a = B[r1 * 3 + col], b = B[r2 * 3 + col];
        double rr = std::sqrt(a * a + b * b);
        double c = 1.0, s = 0.0;
        if (rr > 0) { c = a / rr; s = b / rr; }
        for (int k = 0; k < 3; ++k) {
            double x1 = B[r1 * 3 + k], x2 = B[r2 * 3 + k];
            B[r1 * 3 + k] = c * x1 + s * x2;
            B[r2 * 3 + k] = -s * x1 + c * x2;
        }
        for (int k = 0; k < 3; ++k) {
            double q1 = Q[k * 3 + r1], q2 = Q[k * 3 + r2];
            Q[k * 3 + r1] = c * q1 + s * q2;
            Q[k * 3 + r2] = -s * q1 + c * q2;
        }
    };
    givens(0, 1, 0);
    givens(0, 2, 0);
    givens(1, 2, 1);
    for (int i = 0; i < 9; ++i) U[i] = Q[i];
    for (int i = 0; i < 3; ++i) sig[i] = B[i * 3 + i];
    // make sig0, sig1 non-negative by flipping U columns pairwise with sig2
    for (int i = 0; i < 2; ++i) {
        if (sig[i] < 0) {
            sig[i] = -sig[i];
            sig[2] = -sig[2];
            for (int r = 0; r < 3; ++r) { U[r * 3 + i] = -U[r * 3 + i]; U[r * 3 + 2] = -U[r * 3 + 2]; }
        }
    }
    for (int i = 0; i < 9; ++i) V[i] = Vs[i];
}

// backward_svd, simulation_functions.py:61-87 (clamp :61-67)
inline double clamp_d(double a) { return a >= 0 ? std::max(a, 1e-6) : std::min(a, -1e-6); }

inline void svd3_backward_d(const double gU[9], const double gS[3], const double gV[9], const double U[9],
                            const double sig[3], const double V[9], double gA[9]) {
    double Ut[9], Vt[9], Sg[9] = {0}, gSm[9] = {0};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { Ut[i * 3 + j] = U[j * 3 + i]; Vt[i * 3 + j] = V[j * 3 + i]; }
    for (int i = 0; i < 3; ++i) { Sg[i * 4] = sig[i]; gSm[i * 4] = gS[i]; }
    double t1[9], t2[9], sigma_term[9];
    matmul(U, gSm, t1);
    matmul(t1, Vt, sigma_term);
    double s2[3] = {sig[0] * sig[0], sig[1] * sig[1], sig[2] * sig[2]};
    double f[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) f[i * 3 + j] = (i == j) ? 0.0 : 1.0 / clamp_d(s2[j] - s2[i]);
    // u_term = U ((f * (U^T gU - gU^T U)) S) V^T
    double a1[9], a2[9], gUt[9], gVt[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { gUt[i * 3 + j] = gU[j * 3 + i]; gVt[i * 3 + j] = gV[j * 3 + i]; }
    matmul(Ut, gU, a1);
    matmul(gUt, U, a2);
    double m1[9];
    for (int i = 0; i < 9; ++i) m1[i] = f[i] * (a1[i] - a2[i]);
    double u_term[9];
    matmul(m1, Sg, t1);
    matmul(U, t1, t2);
    matmul(t2, Vt, u_term);
    // v_term = U (S ((f * (V^T gV - gV^T V)) V^T))
    matmul(Vt, gV, a1);
    matmul(gVt, V, a2);
    for (int i = 0; i < 9; ++i) m1[i] = f[i] * (a1[i] - a2[i]);
    double v_term[9];
    matmul(m1, Vt, t1);
    matmul(Sg, t1, t2);
    matmul(U, t2, v_term);
    for (int i = 0; i < 9; ++i) gA[i] = u_term[i] + v_term[i] + sigma_term[i];
}

// ---------------------------------------------------------------------------
// Simulator
// ---------------------------------------------------------------------------
template <class R>
struct Sim {
    DstirSceneDesc d;
    int N, nl, nr, nc, n, G, T, threads;
    R dx, inv_dx, dt;
    R prm[4];
    std::vector<R> traj;     // (T+1)*3
    std::vector<R> st;       // (T+1)*N*NS, states of every step
    std::vector<R> grid;     // T*G*4: momentum xyz + mass after P2G of each step
    std::vector<R> vout;     // G*3 scratch
    std::vector<R> priv;     // threads*G*4 private scatter grids
    std::vector<R> force;    // T*3

    Sim(const DstirSceneDesc& desc, const double* params, const double* trj, int T_, int thr)
        : d(desc), T(T_), threads(std::max(1, thr)) {
        nl = d.n_liquid;
        nr = d.n_rod;
        nc = d.n_container;
        N = nl + nr + nc;
        n = d.n_grid;
        G = n * n * n;
        dx = R(1) / R(n);
        inv_dx = R(n);
        dt = R(d.dt);
        for (int i = 0; i < 4; ++i) prm[i] = R(params[i]);
        traj.resize((size_t)(T + 1) * 3);
        for (size_t i = 0; i < traj.size(); ++i) traj[i] = R(trj[i]);
        st.assign((size_t)(T + 1) * N * NS, R(0));
        grid.assign((size_t)T * G * 4, R(0));
        vout.assign((size_t)G * 3, R(0));
        if (threads > 1) priv.assign((size_t)threads * G * 4, R(0));
        force.assign((size_t)T * 3, R(0));
    }

    inline size_t node(int i, int j, int k) const { return ((size_t)i * n + j) * n + k; }
    R* S(int f, int p) { return &st[((size_t)f * N + p) * NS]; }

    int kind(int p) const { return p < nl ? 0 : (p < nl + nr ? 1 : 2); }

    // base / fx exactly as :106-107 (truncating cast to int)
    static inline bool locate(const R* x, R inv_dx, int n, int base[3], R fx[3]) {
        bool ok = true;
        for (int c = 0; c < 3; ++c) {
            R X = x[c] * inv_dx;
            base[c] = (int)(X - R(0.5));
            fx[c] = X - R(base[c]);
            if (base[c] < 0 || base[c] > n - 3) ok = false;
        }
        return ok;
    }

    // per-particle P2G quantities: mass, velocity to scatter, affine matrix
    void p2g_particle(int f, int p, R& m, R vv[3], R A[9]) {
        R* s = S(f, p);
        int kd = kind(p);
        if (kd == 0) {
            const R* C = s + OC;
            const R* F = s + OF;
            R IC[9], Ft[9];
            for (int i = 0; i < 9; ++i) IC[i] = dt * C[i] + ((i % 4 == 0) ? R(1) : R(0));
            matmul(IC, F, Ft);  // compute_F_tmp :39-42
            R J;
            if (d.j_mode == DSTIR_J_SVD) {
                double Ad[9], U[9], sg[3], V[9];
                for (int i = 0; i < 9; ++i) Ad[i] = (double)Ft[i];
                svd3_d(Ad, U, sg, V);
                J = R(sg[0]) * R(sg[1]) * R(sg[2]);
            } else {
                J = det3(Ft);
            }
            R nrm2 = 0;
            for (int i = 0; i < 9; ++i) nrm2 += C[i] * C[i];
            R gamma = std::sqrt(nrm2) + R(1e-6);
            Visc<R> vs = viscosity<R>(d.model, prm, gamma);
            R k = R(d.bulk_modulus);
            R pr = (k / R(2)) * (J - (R(1) / J) - R(1)) * J;
            R alpha = (-dt * R(d.liquid_p_vol) * R(4) * inv_dx * inv_dx);
            m = R(d.liquid_p_mass);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    R Dab = R(0.5) * (C[a * 3 + b] + C[b * 3 + a]);
                    R sig = vs.eta * Dab + ((a == b) ? pr : R(0));
                    A[a * 3 + b] = alpha * sig + m * C[a * 3 + b];
                }
            vv[0] = s[OV + 0];
            vv[1] = s[OV + 1] + dt * R(d.gravity);
            vv[2] = s[OV + 2];
            R* Fn = S(f + 1, p) + OF;  // F[f+1] = F_tmp (:153)
            for (int i = 0; i < 9; ++i) Fn[i] = Ft[i];
        } else {
            m = R(kd == 1 ? d.rod_p_mass : d.container_p_mass);
            for (int i = 0; i < 9; ++i) A[i] = m * s[OC + i];
            for (int c = 0; c < 3; ++c) vv[c] = s[OV + c];
        }
    }

    void scatter_particle(int f, int p, R* g, uint32_t& status) {
        R m, vv[3], A[9];
        p2g_particle(f, p, m, vv, A);
        int base[3];
        R fx[3], w[3][3], dw[3][3];
        if (!locate(S(f, p) + OX, inv_dx, n, base, fx)) { status |= DSTIR_STATUS_OUT_OF_GRID; return; }
        bspline(fx, w, dw);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    R dpos[3] = {(R(i) - fx[0]) * dx, (R(j) - fx[1]) * dx, (R(k) - fx[2]) * dx};
                    R W = w[i][0] * w[j][1] * w[k][2];
                    R* gn = g + node(base[0] + i, base[1] + j, base[2] + k) * 4;
                    for (int a = 0; a < 3; ++a) {
                        R ad = A[a * 3 + 0] * dpos[0] + A[a * 3 + 1] * dpos[1] + A[a * 3 + 2] * dpos[2];
                        gn[a] += W * (m * vv[a] + ad);
                    }
                    gn[3] += W * m;
                }
    }

    // parallel scatter helper: fn(p, grid) for p in [0,N), results summed into out (G*4)
    template <class Fn>
    void scatter_all(R* out, Fn fn) {
        if (threads == 1) {
            for (int p = 0; p < N; ++p) fn(p, out);
            return;
        }
        std::fill(priv.begin(), priv.end(), R(0));
#pragma omp parallel num_threads(threads)
        {
#ifdef _OPENMP
            int t = omp_get_thread_num();
#else
            int t = 0;
#endif
            int lo = (int)((int64_t)N * t / threads), hi = (int)((int64_t)N * (t + 1) / threads);
            R* g = &priv[(size_t)t * G * 4];
            for (int p = lo; p < hi; ++p) fn(p, g);
        }
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t q = 0; q < (int64_t)G * 4; ++q) {
            R s = out[q];
            for (int t = 0; t < threads; ++t) s += priv[(size_t)t * G * 4 + q];
            out[q] = s;
        }
    }

    // grid_op :199-225 (+ cylinder rod), returns the reaction force for the cylinder
    void grid_op(int f, const R* g, R* vo, R frc[3]) {
        R fsum[3] = {0, 0, 0};
        R rodv[3], rc[3];
        for (int c = 0; c < 3; ++c) {
            rc[c] = traj[(size_t)f * 3 + c];
            rodv[c] = (traj[(size_t)(f + 1) * 3 + c] - traj[(size_t)f * 3 + c]) / dt;
        }
        bool cyl = d.rod_mode == DSTIR_ROD_CYLINDER;
        // serial over nodes for a deterministic force sum; parallel otherwise
        auto body = [&](size_t idx, R* fs) {
            int i = (int)(idx / ((size_t)n * n)), j = (int)((idx / n) % n), k = (int)(idx % n);
            const R* gn = g + idx * 4;
            R inv_m = R(1) / (gn[3] + R(1e-10));
            R v[3] = {inv_m * gn[0], inv_m * gn[1], inv_m * gn[2]};
            const bool massive = gn[3] > R(0);
            if (massive) BRANCH(7);
            if (d.container_wall) {
                R r = R(d.container_r);
                R dist[3] = {R(i) * dx - R(d.container_cx), R(0), R(k) * dx - R(d.container_cz)};
                R n2 = dist[0] * dist[0] + dist[2] * dist[2];
                if (n2 > r * r) {
                    R nn = std::sqrt(n2);
                    R u0 = dist[0] / nn, u2 = dist[2] / nn;
                    R dot = v[0] * u0 + v[2] * u2;
                    v[0] -= u0 * dot;
                    v[2] -= u2 * dot;
                    if (massive && dot != R(0)) BRANCH(0);
                }
            }
            int b = d.bound;
            if (i < b && v[0] < 0) { v[0] = 0; if (massive) BRANCH(1); }
            if (i > n - b && v[0] > 0) { v[0] = 0; if (massive) BRANCH(2); }
            if (k < b && v[2] < 0) { v[2] = 0; if (massive) BRANCH(3); }
            if (k > n - b && v[2] > 0) { v[2] = 0; if (massive) BRANCH(4); }
            if (j < b && v[1] < 0) { v[1] = 0; if (massive) BRANCH(5); }
#ifdef ORACLE_CONTINUOUS_TOP
            // diagnostic build: a plain clamp instead of the sticky top
            if (j > n - b && v[1] > 0) v[1] = 0;
#else
            if (j > n - b && v[1] > 0) {  // sticky top, :221-224
                v[0] = 0; v[1] = 0; v[2] = 0;
                if (massive) BRANCH(6);
            }
#endif
            if (cyl) {
                R ddx = R(i) * dx - rc[0], ddz = R(k) * dx - rc[2];
                R rr = R(d.rod_radius);
                if (ddx * ddx + ddz * ddz < rr * rr && R(j) * dx >= rc[1]) {
                    for (int c = 0; c < 3; ++c) {
                        R u = inv_m * gn[c];
                        fs[c] += gn[3] * (rodv[c] - u) / dt;
                        v[c] = rodv[c];
                    }
                }
            }
            for (int c = 0; c < 3; ++c) vo[idx * 3 + c] = v[c];
        };
        if (cyl || threads == 1) {
            for (size_t idx = 0; idx < (size_t)G; ++idx) body(idx, fsum);
        } else {
#pragma omp parallel for num_threads(threads) schedule(static)
            for (int64_t idx = 0; idx < (int64_t)G; ++idx) {
                R dummy[3];
                body((size_t)idx, dummy);
            }
        }
        for (int c = 0; c < 3; ++c) frc[c] = fsum[c];
    }

    // g2p :228-290 for particle p, returns rod dv in dv (particle rod only)
    void g2p_particle(int f, int p, const R* vo, R dv[3], uint32_t& status) {
        R* s = S(f, p);
        R* sn = S(f + 1, p);
        int base[3];
        R fx[3], w[3][3], dw[3][3];
        R nv[3] = {0, 0, 0}, nC[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        bool ok = locate(s + OX, inv_dx, n, base, fx);
        if (!ok) status |= DSTIR_STATUS_OUT_OF_GRID;
        if (ok) {
            bspline(fx, w, dw);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k) {
                        R dp[3] = {R(i) - fx[0], R(j) - fx[1], R(k) - fx[2]};
                        const R* gv = vo + node(base[0] + i, base[1] + j, base[2] + k) * 3;
                        R W = w[i][0] * w[j][1] * w[k][2];
                        for (int a = 0; a < 3; ++a) {
                            nv[a] += W * gv[a];
                            for (int b2 = 0; b2 < 3; ++b2) nC[a * 3 + b2] += R(4) * W * (gv[a] * dp[b2]) * inv_dx;
                        }
                    }
        }
        int kd = kind(p);
        for (int i = 0; i < 9; ++i) sn[OC + i] = nC[i];
        if (kd == 0) {
            for (int c = 0; c < 3; ++c) {
                sn[OV + c] = nv[c];
                sn[OX + c] = s[OX + c] + dt * nv[c];
            }
            for (int i = 0; i < NS; ++i)
                if (!std::isfinite((double)sn[i])) status |= DSTIR_STATUS_NAN;
        } else if (kd == 1) {
            for (int c = 0; c < 3; ++c) {
                R tv = (traj[(size_t)(f + 1) * 3 + c] - traj[(size_t)f * 3 + c]) / dt;
                dv[c] = tv - nv[c];
                sn[OV + c] = tv;
                sn[OX + c] = s[OX + c] + tv * dt;
            }
        } else {
            for (int c = 0; c < 3; ++c) {
                sn[OV + c] = R(0);
                sn[OX + c] = s[OX + c];
            }
        }
    }

    uint32_t step(int f) {
        uint32_t status = 0;
        R* g = &grid[(size_t)f * G * 4];
        std::fill(g, g + (size_t)G * 4, R(0));
        // liquid F_tmp / stress / F[f+1] are written inside p2g_particle
        if (threads == 1) {
            for (int p = 0; p < N; ++p) scatter_particle(f, p, g, status);
        } else {
            std::vector<uint32_t> sts(threads, 0);
            scatter_all(g, [&](int p, R* gg) {
#ifdef _OPENMP
                int t = omp_get_thread_num();
#else
                int t = 0;
#endif
                scatter_particle(f, p, gg, sts[t]);
            });
            for (auto s2 : sts) status |= s2;
        }
        R frc[3];
        grid_op(f, g, vout.data(), frc);
        // g2p; the rod dv sum is taken in particle order
        std::vector<R> dvs((size_t)std::max(nr, 1) * 3, R(0));
        std::vector<uint32_t> sts(threads, 0);
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int p = 0; p < N; ++p) {
#ifdef _OPENMP
            int t = omp_get_thread_num();
#else
            int t = 0;
#endif
            R dv[3] = {0, 0, 0};
            g2p_particle(f, p, vout.data(), dv, sts[t]);
            if (kind(p) == 1)
                for (int c = 0; c < 3; ++c) dvs[(size_t)(p - nl) * 3 + c] = dv[c];
        }
        for (auto s2 : sts) status |= s2;
        // carry F of rod/container particles (unused) forward unchanged
        for (int p = nl; p < N; ++p)
            for (int i = 0; i < 9; ++i) S(f + 1, p)[OF + i] = S(f, p)[OF + i];
        if (d.rod_mode == DSTIR_ROD_PARTICLES) {
            R tot[3] = {0, 0, 0};
            for (int p = 0; p < nr; ++p)
                for (int c = 0; c < 3; ++c) tot[c] += dvs[(size_t)p * 3 + c];
            for (int c = 0; c < 3; ++c) force[(size_t)f * 3 + c] = tot[c] * R(d.force_scale);
        } else {
            for (int c = 0; c < 3; ++c) force[(size_t)f * 3 + c] = frc[c];
        }
        return status;
    }

    uint32_t rollout() {
        uint32_t status = 0;
        for (int f = 0; f < T; ++f) status |= step(f);
        return status;
    }

    // -----------------------------------------------------------------------
    // adjoint
    // -----------------------------------------------------------------------
    std::vector<R> adj_next, adj_cur;  // N*NS each
    std::vector<R> gadj;               // G*4 grid adjoint (velocity-out adjoint, then P/M adjoint)
    std::vector<R> gpm;                // G*4 P/M adjoint
    double dprm[4] = {0, 0, 0, 0};

    // dL_dstateT (optional): adjoint of the final state, for chaining the
    // reverse pass over consecutive segments of a long rollout
    void backward(const double* dL_dforce, double* dL_dparams, double* dL_dstate0,
                  const double* dL_dstateT = nullptr) {
        adj_next.assign((size_t)N * NS, R(0));
        if (dL_dstateT)
            for (size_t i = 0; i < (size_t)N * NS; ++i) adj_next[i] = R(dL_dstateT[i]);
        adj_cur.assign((size_t)N * NS, R(0));
        gadj.assign((size_t)G * 4, R(0));
        gpm.assign((size_t)G * 4, R(0));
        for (int i = 0; i < 4; ++i) dprm[i] = 0;
        for (int f = T - 1; f >= 0; --f) {
            R fbar[3];
            for (int c = 0; c < 3; ++c) fbar[c] = R(dL_dforce[(size_t)f * 3 + c]);
            const R* g = &grid[(size_t)f * G * 4];
            R frc[3];
            grid_op(f, g, vout.data(), frc);  // recompute v_out of step f
            std::fill(adj_cur.begin(), adj_cur.end(), R(0));
            // (1) G2P adjoint: scatter into gadj (velocity-out adjoint)
            std::fill(gadj.begin(), gadj.end(), R(0));
            auto g2p_adj = [&](int p, R* ga) { g2p_adj_particle(f, p, fbar, ga); };
            scatter_all(gadj.data(), g2p_adj);
            // (2) grid adjoint
            grid_adj(f, g, fbar);
            // (3) P2G adjoint (gather)
            std::vector<double> part((size_t)threads * 4, 0.0);
#pragma omp parallel for num_threads(threads) schedule(static)
            for (int p = 0; p < N; ++p) {
#ifdef _OPENMP
                int t = omp_get_thread_num();
#else
                int t = 0;
#endif
                double pp[4] = {0, 0, 0, 0};
                p2g_adj_particle(f, p, pp);
                for (int i = 0; i < 4; ++i) part[(size_t)t * 4 + i] += pp[i];
            }
            for (int t = 0; t < threads; ++t)
                for (int i = 0; i < 4; ++i) dprm[i] += part[(size_t)t * 4 + i];
            std::swap(adj_next, adj_cur);
        }
        for (int i = 0; i < 4; ++i) dL_dparams[i] = dprm[i];
        if (dL_dstate0)
            for (size_t i = 0; i < (size_t)N * NS; ++i) dL_dstate0[i] = (double)adj_next[i];
    }

    void g2p_adj_particle(int f, int p, const R fbar[3], R* ga) {
        R* s = S(f, p);
        const R* an = &adj_next[(size_t)p * NS];
        R* ac = &adj_cur[(size_t)p * NS];
        int kd = kind(p);
        int base[3];
        R fx[3], w[3][3], dw[3][3];
        if (!locate(s + OX, inv_dx, n, base, fx)) return;
        bspline(fx, w, dw);
        R vnb[3];
        const R* Cb = an + OC;
        if (kd == 0) {
            for (int c = 0; c < 3; ++c) {
                vnb[c] = an[OV + c] + dt * an[OX + c];
                ac[OX + c] += an[OX + c];
            }
        } else if (kd == 1) {
            R sc = (d.rod_mode == DSTIR_ROD_PARTICLES) ? R(d.force_scale) : R(0);
            for (int c = 0; c < 3; ++c) vnb[c] = -fbar[c] * sc;
        } else {
            for (int c = 0; c < 3; ++c) vnb[c] = 0;
        }
        R fxb[3] = {0, 0, 0};
        R c4 = R(4) * inv_dx;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    int o[3] = {i, j, k};
                    R dp[3] = {R(i) - fx[0], R(j) - fx[1], R(k) - fx[2]};
                    size_t nd = node(base[0] + i, base[1] + j, base[2] + k);
                    const R* gv = &vout[nd * 3];
                    R W = w[i][0] * w[j][1] * w[k][2];
                    R Wb = 0;
                    R* gg = ga + nd * 4;
                    for (int a = 0; a < 3; ++a) {
                        R Cd = Cb[a * 3 + 0] * dp[0] + Cb[a * 3 + 1] * dp[1] + Cb[a * 3 + 2] * dp[2];
                        gg[a] += W * vnb[a] + c4 * W * Cd;
                        Wb += vnb[a] * gv[a] + c4 * gv[a] * Cd;
                    }
                    if (kd == 0) {
                        // d dp_b = -d fx_b ; dC/d dp_b = c4 W g_a Cb_ab
                        for (int b2 = 0; b2 < 3; ++b2) {
                            R s2 = 0;
                            for (int a = 0; a < 3; ++a) s2 += Cb[a * 3 + b2] * gv[a];
                            fxb[b2] -= c4 * W * s2;
                        }
                        fxb[0] += Wb * dw[o[0]][0] * w[o[1]][1] * w[o[2]][2];
                        fxb[1] += Wb * w[o[0]][0] * dw[o[1]][1] * w[o[2]][2];
                        fxb[2] += Wb * w[o[0]][0] * w[o[1]][1] * dw[o[2]][2];
                    }
                }
        if (kd == 0)
            for (int c = 0; c < 3; ++c) ac[OX + c] += inv_dx * fxb[c];
    }

    void grid_adj(int f, const R* g, const R fbar[3]) {
        R rodv[3], rc[3];
        for (int c = 0; c < 3; ++c) {
            rc[c] = traj[(size_t)f * 3 + c];
            rodv[c] = (traj[(size_t)(f + 1) * 3 + c] - traj[(size_t)f * 3 + c]) / dt;
        }
        bool cyl = d.rod_mode == DSTIR_ROD_CYLINDER;
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t idx = 0; idx < (int64_t)G; ++idx) {
            int i = (int)(idx / ((int64_t)n * n)), j = (int)((idx / n) % n), k = (int)(idx % n);
            const R* gn = g + idx * 4;
            const R* vb = &gadj[idx * 4];
            R inv_m = R(1) / (gn[3] + R(1e-10));
            R u[3] = {inv_m * gn[0], inv_m * gn[1], inv_m * gn[2]};
            R v[3] = {u[0], u[1], u[2]};
            bool proj = false;
            R u0 = 0, u2 = 0;
            if (d.container_wall) {
                R r = R(d.container_r);
                R dist[3] = {R(i) * dx - R(d.container_cx), R(0), R(k) * dx - R(d.container_cz)};
                R n2 = dist[0] * dist[0] + dist[2] * dist[2];
                if (n2 > r * r) {
                    R nn = std::sqrt(n2);
                    u0 = dist[0] / nn;
                    u2 = dist[2] / nn;
                    R dot = v[0] * u0 + v[2] * u2;
                    v[0] -= u0 * dot;
                    v[2] -= u2 * dot;
                    proj = true;
                }
            }
            R mask[3] = {1, 1, 1};
            int b = d.bound;
            if (i < b && v[0] < 0) { v[0] = 0; mask[0] = 0; }
            if (i > n - b && v[0] > 0) { v[0] = 0; mask[0] = 0; }
            if (k < b && v[2] < 0) { v[2] = 0; mask[2] = 0; }
            if (k > n - b && v[2] > 0) { v[2] = 0; mask[2] = 0; }
            if (j < b && v[1] < 0) { v[1] = 0; mask[1] = 0; }
#ifdef ORACLE_CONTINUOUS_TOP
            if (j > n - b && v[1] > 0) { v[1] = 0; mask[1] = 0; }
#else
            if (j > n - b && v[1] > 0) { mask[0] = mask[1] = mask[2] = 0; }
#endif
            R ub[3];
            R mb = 0;
            bool inside = false;
            if (cyl) {
                R ddx = R(i) * dx - rc[0], ddz = R(k) * dx - rc[2];
                R rr = R(d.rod_radius);
                inside = (ddx * ddx + ddz * ddz < rr * rr && R(j) * dx >= rc[1]);
            }
            if (inside) {
                for (int c = 0; c < 3; ++c) {
                    ub[c] = -gn[3] * fbar[c] / dt;
                    mb += fbar[c] * (rodv[c] - u[c]) / dt;
                }
            } else {
                R vb2[3] = {mask[0] * vb[0], mask[1] * vb[1], mask[2] * vb[2]};
                if (proj) {
                    R dot = vb2[0] * u0 + vb2[2] * u2;
                    vb2[0] -= u0 * dot;
                    vb2[2] -= u2 * dot;
                }
                for (int c = 0; c < 3; ++c) ub[c] = vb2[c];
            }
            R Pu = 0;
            for (int c = 0; c < 3; ++c) Pu += gn[c] * ub[c];
            R* out = &gpm[idx * 4];
            for (int c = 0; c < 3; ++c) out[c] = inv_m * ub[c];
            out[3] = mb - inv_m * inv_m * Pu;
        }
    }

    void p2g_adj_particle(int f, int p, double pp[4]) {
        R* s = S(f, p);
        R* ac = &adj_cur[(size_t)p * NS];
        const R* an = &adj_next[(size_t)p * NS];
        int kd = kind(p);
        int base[3];
        R fx[3], w[3][3], dw[3][3];
        bool ok = locate(s + OX, inv_dx, n, base, fx);
        // recompute the P2G quantities (without rewriting F[f+1])
        const R* C = s + OC;
        const R* F = s + OF;
        R m, vv[3], A[9];
        R Ft[9], IC[9], J = 0, gamma = 0, nrm = 0, pr = 0, alpha = 0;
        Visc<R> vs{};
        double U[9], sg[3], V[9];
        if (kd == 0) {
            for (int i = 0; i < 9; ++i) IC[i] = dt * C[i] + ((i % 4 == 0) ? R(1) : R(0));
            matmul(IC, F, Ft);
            if (d.j_mode == DSTIR_J_SVD) {
                double Ad[9];
                for (int i = 0; i < 9; ++i) Ad[i] = (double)Ft[i];
                svd3_d(Ad, U, sg, V);
                J = R(sg[0]) * R(sg[1]) * R(sg[2]);
            } else {
                J = det3(Ft);
            }
            R nrm2 = 0;
            for (int i = 0; i < 9; ++i) nrm2 += C[i] * C[i];
            nrm = std::sqrt(nrm2);
            gamma = nrm + R(1e-6);
            vs = viscosity<R>(d.model, prm, gamma);
            R k = R(d.bulk_modulus);
            pr = (k / R(2)) * (J - (R(1) / J) - R(1)) * J;
            alpha = (-dt * R(d.liquid_p_vol) * R(4) * inv_dx * inv_dx);
            m = R(d.liquid_p_mass);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    R Dab = R(0.5) * (C[a * 3 + b] + C[b * 3 + a]);
                    A[a * 3 + b] = alpha * (vs.eta * Dab + ((a == b) ? pr : R(0))) + m * C[a * 3 + b];
                }
            vv[0] = s[OV + 0];
            vv[1] = s[OV + 1] + dt * R(d.gravity);
            vv[2] = s[OV + 2];
        } else {
            m = R(kd == 1 ? d.rod_p_mass : d.container_p_mass);
            for (int i = 0; i < 9; ++i) A[i] = m * C[i];
            for (int c = 0; c < 3; ++c) vv[c] = s[OV + c];
        }
        R Ab[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vvb[3] = {0, 0, 0}, fxb[3] = {0, 0, 0};
        if (ok) {
            bspline(fx, w, dw);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k) {
                        int o[3] = {i, j, k};
                        R dpos[3] = {(R(i) - fx[0]) * dx, (R(j) - fx[1]) * dx, (R(k) - fx[2]) * dx};
                        R W = w[i][0] * w[j][1] * w[k][2];
                        const R* gb = &gpm[node(base[0] + i, base[1] + j, base[2] + k) * 4];
                        R Wb = gb[3] * m;
                        for (int a = 0; a < 3; ++a) {
                            R ad = A[a * 3 + 0] * dpos[0] + A[a * 3 + 1] * dpos[1] + A[a * 3 + 2] * dpos[2];
                            Wb += gb[a] * (m * vv[a] + ad);
                            vvb[a] += W * m * gb[a];
                            for (int b2 = 0; b2 < 3; ++b2) Ab[a * 3 + b2] += W * gb[a] * dpos[b2];
                        }
                        if (kd == 0) {
                            for (int b2 = 0; b2 < 3; ++b2) {
                                R s2 = 0;
                                for (int a = 0; a < 3; ++a) s2 += A[a * 3 + b2] * gb[a];
                                fxb[b2] -= W * s2 * dx;
                            }
                            fxb[0] += Wb * dw[o[0]][0] * w[o[1]][1] * w[o[2]][2];
                            fxb[1] += Wb * w[o[0]][0] * dw[o[1]][1] * w[o[2]][2];
                            fxb[2] += Wb * w[o[0]][0] * w[o[1]][1] * dw[o[2]][2];
                        }
                    }
        }
        if (kd != 0) {
            for (int i = 0; i < 9; ++i) ac[OC + i] += m * Ab[i];
            return;
        }
        for (int c = 0; c < 3; ++c) {
            ac[OX + c] += inv_dx * fxb[c];
            ac[OV + c] += vvb[c];
        }
        // A = alpha*sigma + m*C
        R sigb[9];
        for (int i = 0; i < 9; ++i) {
            ac[OC + i] += m * Ab[i];
            sigb[i] = alpha * Ab[i];
        }
        // sigma = eta*D + pr*I
        R etab = 0, trb = sigb[0] + sigb[4] + sigb[8];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                R Dab = R(0.5) * (C[a * 3 + b] + C[b * 3 + a]);
                etab += sigb[a * 3 + b] * Dab;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                ac[OC + a * 3 + b] += vs.eta * R(0.5) * (sigb[a * 3 + b] + sigb[b * 3 + a]);
        R k = R(d.bulk_modulus);
        R Jb = trb * (k / R(2)) * (R(2) * J - R(1));
        // F_tmp adjoint: from F[f+1] = F_tmp and from J
        R Ftb[9];
        for (int i = 0; i < 9; ++i) Ftb[i] = an[OF + i];
        if (d.j_mode == DSTIR_J_SVD) {
            double gS[3] = {(double)Jb * sg[1] * sg[2], (double)Jb * sg[0] * sg[2], (double)Jb * sg[0] * sg[1]};
            double z[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, gA[9];
            svd3_backward_d(z, gS, z, U, sg, V, gA);
            for (int i = 0; i < 9; ++i) Ftb[i] += R(gA[i]);
        } else {
            R cf[9];
            cof3(Ft, cf);
            for (int i = 0; i < 9; ++i) Ftb[i] += Jb * cf[i];
        }
        // viscosity
        R gammab = etab * vs.deta_dgamma;
        for (int i = 0; i < 4; ++i) pp[i] += (double)(etab * vs.deta_dp[i]);
        if (nrm > R(0))
            for (int i = 0; i < 9; ++i) ac[OC + i] += gammab * C[i] / nrm;
        // F_tmp = (I + dt C) F
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                R sF = 0, sC = 0;
                for (int c = 0; c < 3; ++c) {
                    sF += IC[c * 3 + a] * Ftb[c * 3 + b];  // (IC^T Ftb)_ab
                    sC += Ftb[a * 3 + c] * F[b * 3 + c];   // (Ftb F^T)_ab
                }
                ac[OF + a * 3 + b] += sF;
                ac[OC + a * 3 + b] += dt * sC;
            }
    }
};

template <class R>
void load_state0(Sim<R>& sim, const double* x0, const double* v0, const double* C0, const double* F0) {
    for (int p = 0; p < sim.N; ++p) {
        R* s = sim.S(0, p);
        for (int c = 0; c < 3; ++c) {
            s[OX + c] = R(x0[(size_t)p * 3 + c]);
            s[OV + c] = v0 ? R(v0[(size_t)p * 3 + c]) : R(0);
        }
        for (int i = 0; i < 9; ++i) {
            s[OC + i] = C0 ? R(C0[(size_t)p * 9 + i]) : R(0);
            s[OF + i] = F0 ? R(F0[(size_t)p * 9 + i]) : ((i % 4 == 0) ? R(1) : R(0));
        }
    }
}

template <class R>
int rollout_impl(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                 const double* x0, const double* v0, const double* C0, const double* F0,
                 double* force_out, double* states_out, int threads, const double* dL_dforce,
                 double* dL_dparams, double* dL_dstate0, const double* dL_dstateT = nullptr,
                 double* last_out = nullptr) {
    if (!d || !params || !traj || !x0 || T < 0) return DSTIR_EINVAL;
    if (d->n_grid < 4) return DSTIR_EINVAL;
    Sim<R> sim(*d, params, traj, T, threads);
    load_state0(sim, x0, v0, C0, F0);
    uint32_t status = sim.rollout();
    if (force_out)
        for (size_t i = 0; i < (size_t)T * 3; ++i) force_out[i] = (double)sim.force[i];
    if (states_out)
        for (size_t i = 0; i < sim.st.size(); ++i) states_out[i] = (double)sim.st[i];
    if (last_out)
        for (size_t i = 0; i < (size_t)sim.N * NS; ++i) last_out[i] = (double)sim.st[(size_t)T * sim.N * NS + i];
    if (dL_dforce) sim.backward(dL_dforce, dL_dparams, dL_dstate0, dL_dstateT);
    return (int)status;
}

}  // namespace

extern "C" {

// Forward rollout of T substeps. Returns the OR of DSTIR_STATUS_* bits (>= 0)
// or a negative DSTIR_E* code.  force_out [T,3]; states_out [(T+1),N,24] or NULL.
int oracle_rollout_f64(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                       const double* x0, const double* v0, const double* C0, const double* F0,
                       double* force_out, double* states_out, int threads) {
    return rollout_impl<double>(d, params, traj, T, x0, v0, C0, F0, force_out, states_out, threads,
                                nullptr, nullptr, nullptr);
}
int oracle_rollout_f32(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                       const double* x0, const double* v0, const double* C0, const double* F0,
                       double* force_out, double* states_out, int threads) {
    return rollout_impl<float>(d, params, traj, T, x0, v0, C0, F0, force_out, states_out, threads,
                               nullptr, nullptr, nullptr);
}
// Forward rollout plus the reverse pass for dL/dforce [T,3]:
// dL_dparams [4], dL_dstate0 [N,24] (or NULL).
int oracle_grad_f64(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                    const double* x0, const double* v0, const double* C0, const double* F0,
                    const double* dL_dforce, double* force_out, double* dL_dparams, double* dL_dstate0,
                    int threads) {
    if (!dL_dforce || !dL_dparams) return DSTIR_EINVAL;
    return rollout_impl<double>(d, params, traj, T, x0, v0, C0, F0, force_out, nullptr, threads,
                                dL_dforce, dL_dparams, dL_dstate0);
}
int oracle_grad_f32(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                    const double* x0, const double* v0, const double* C0, const double* F0,
                    const double* dL_dforce, double* force_out, double* dL_dparams, double* dL_dstate0,
                    int threads) {
    if (!dL_dforce || !dL_dparams) return DSTIR_EINVAL;
    return rollout_impl<float>(d, params, traj, T, x0, v0, C0, F0, force_out, nullptr, threads,
                               dL_dforce, dL_dparams, dL_dstate0);
}

// Segment forms for rollouts too long to keep every state: the rollout
// returns only its final state [N,24]; the reverse pass also takes the
// adjoint of the final state [N,24] (NULL: zero).
int oracle_rollout_last_f64(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                            const double* x0, const double* v0, const double* C0, const double* F0,
                            double* force_out, double* last_out, int threads) {
    return rollout_impl<double>(d, params, traj, T, x0, v0, C0, F0, force_out, nullptr, threads, nullptr,
                                nullptr, nullptr, nullptr, last_out);
}
int oracle_grad_seeded_f64(const DstirSceneDesc* d, const double* params, const double* traj, int T,
                           const double* x0, const double* v0, const double* C0, const double* F0,
                           const double* dL_dforce, const double* dL_dstateT, double* force_out,
                           double* dL_dparams, double* dL_dstate0, int threads) {
    if (!dL_dforce || !dL_dparams) return DSTIR_EINVAL;
    return rollout_impl<double>(d, params, traj, T, x0, v0, C0, F0, force_out, nullptr, threads, dL_dforce,
                                dL_dparams, dL_dstate0, dL_dstateT);
}

void oracle_svd3_f64(const double* A, double* U, double* S, double* V, int64_t n) {
    for (int64_t i = 0; i < n; ++i) svd3_d(A + i * 9, U + i * 9, S + i * 3, V + i * 9);
}

void oracle_svd3_backward_f64(const double* gU, const double* gS, const double* gV, const double* U,
                              const double* S, const double* V, double* gA, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        svd3_backward_d(gU + i * 9, gS + i * 3, gV + i * 9, U + i * 9, S + i * 3, V + i * 9, gA + i * 9);
}

#ifdef ORACLE_BRANCH_COUNTS
// Copies the branch counters (NBRANCH entries, see g_branch) to out, up to n
// of them, and clears them; returns NBRANCH.
int oracle_branch_counts(long long* out, int n) {
    for (int i = 0; i < NBRANCH; ++i) {
        if (out && i < n) out[i] = g_branch[i];
        g_branch[i] = 0;
    }
    return NBRANCH;
}
#endif

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
