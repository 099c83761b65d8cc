// solver_oracle.cpp -- CPU restatement of the reference's implicit-solver
// components (TEST INFRASTRUCTURE ONLY: the checker for the GPU solvers).
//
//   level geometry  3_5/ModMultigrid.f90:97-233 (iGeometry = 1)
//   PFSS operator   3_5/ModPFSS.f90:21-100 (level 1)
//   1-layer halo    3_5/ModGC.f90:53-76,174-284 (face ghosts, grouped per source
//                   in first-appearance order, i-j-k loop order) and the
//                   interpolation of 3_5/ModMath.f90:208-248
//   SpMV            3_5/ModLinearSolver.f90:34-51
//   V-cycle parts   restriction 3_6/ModMath.f90:353-368, prolongation
//                   3_6/ModMath.f90:370-384, the smoother's cell update
//                   3_5/ModMultigrid.f90:316-324 (FP32, for component parity)
//   MG-PCG          3_5/ModLinearSolver.f90:201-427 as the GPU corrects it
//                   (FP64 throughout: the CPU reference solve of a batch)
// The reference solver runs in default real (FP32); the SpMV and the CPU
// solve keep its operation order and evaluate in FP64, the precision in which
// the GPU solve judges convergence.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

// The tree of the oracle (falcon_oracle.cpp) is reused through these hooks.
extern "C" int orc_num_blocks(void* h, int32_t* nb, int32_t* nyin);
extern "C" int orc_block_ranges(void* h, double* out);
extern "C" int orc_block_flags(void* h, int32_t* out);
extern "C" int orc_find_leaf(void* h, const double* rtp, int32_t yin);
extern "C" void orc_coord_conv(const double* in, double* out);

namespace {

struct Geo {
    int m;
    std::vector<double> xI[3], xF[3];
    double dx[3];
    void init(const double* rng, int mm) {   // rng[3][2]
        m = mm;
        for (int d = 0; d < 3; ++d) {
            const double r1 = rng[2 * d], r2 = rng[2 * d + 1];
            xI[d].resize(m + 2);
            xF[d].resize(m + 2);
            for (int i = 0; i <= m + 1; ++i)
                xI[d][i] = (r1 * (double)((float)(m - i) + 0.5f) + r2 * (double)((float)i - 0.5f)) / m;
            for (int i = 1; i <= m + 1; ++i) xF[d][i] = (r1 * (double)(m + 1 - i) + r2 * (double)(i - 1)) / m;
            dx[d] = (r2 - r1) / m;
        }
    }
};

inline size_t fidx_i(int m, int b, int i, int j, int k) { return (((size_t)b * m + (k - 1)) * m + (j - 1)) * (m + 1) + (i - 1); }
inline size_t fidx_j(int m, int b, int i, int j, int k) { return (((size_t)b * m + (k - 1)) * (m + 1) + (j - 1)) * m + (i - 1); }
inline size_t fidx_k(int m, int b, int i, int j, int k) { return (((size_t)b * (m + 1) + (k - 1)) * m + (j - 1)) * m + (i - 1); }
inline size_t cidx(int m, int b, int i, int j, int k) { return (((size_t)b * m + (k - 1)) * m + (j - 1)) * m + (i - 1); }

}  // namespace

extern "C" {

// PFSS face-coefficient operator on level-1 grids with m cells per block edge
int orc_pfss_operator(void* h, int32_t m, double* Aii, double* Ai, double* Aj, double* Ak) {
    int32_t nb, ny;
    orc_num_blocks(h, &nb, &ny);
    std::vector<double> rng((size_t)nb * 6);
    std::vector<int32_t> fl(nb);
    orc_block_ranges(h, rng.data());
    orc_block_flags(h, fl.data());
    for (int b = 0; b < nb; ++b) {
        Geo G;
        G.init(&rng[(size_t)b * 6], m);
        const std::vector<double>&xiI = G.xI[0], &xjI = G.xI[1], &xiF = G.xF[0], &xjF = G.xF[1], &xkF = G.xF[2];
        // MGL1%Ai_FLL=-MGL1%Si_FLL/MGL1%Di_FLL etc. (3_5/ModPFSS.f90:64-66)
        for (int k = 1; k <= m; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= m + 1; ++i) {
                    const double S = xiF[i] * xiF[i] * (std::cos(xjF[j]) - std::cos(xjF[j + 1])) * (xkF[k + 1] - xkF[k]);
                    Ai[fidx_i(m, b, i, j, k)] = -S / G.dx[0];
                }
        for (int k = 1; k <= m; ++k)
            for (int j = 1; j <= m + 1; ++j)
                for (int i = 1; i <= m; ++i) {
                    const double S = 0.5 * (xiF[i + 1] * xiF[i + 1] - xiF[i] * xiF[i]) * (xkF[k + 1] - xkF[k]) * std::sin(xjF[j]);
                    Aj[fidx_j(m, b, i, j, k)] = -S / (xiI[i] * G.dx[1]);
                }
        for (int k = 1; k <= m + 1; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= m; ++i) {
                    const double S = 0.5 * (xiF[i + 1] * xiF[i + 1] - xiF[i] * xiF[i]) * (xjF[j + 1] - xjF[j]);
                    Ak[fidx_k(m, b, i, j, k)] = -S / (xiI[i] * G.dx[2] * std::sin(xjI[j]));
                }
        const bool top = fl[b] & 2, bottom = fl[b] & 4;
        if (bottom)
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j) Ai[fidx_i(m, b, 1, j, k)] = 0.0;
        for (int k = 1; k <= m; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= m; ++i)
                    Aii[cidx(m, b, i, j, k)] =
                        -(Ai[fidx_i(m, b, i, j, k)] + Ai[fidx_i(m, b, i + 1, j, k)] + Aj[fidx_j(m, b, i, j, k)] +
                          Aj[fidx_j(m, b, i, j + 1, k)] + Ak[fidx_k(m, b, i, j, k)] + Ak[fidx_k(m, b, i, j, k + 1)]);
        if (top)
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j) {
                    Aii[cidx(m, b, m, j, k)] = Aii[cidx(m, b, m, j, k)] - Ai[fidx_i(m, b, m + 1, j, k)];
                    Ai[fidx_i(m, b, m + 1, j, k)] = 0.0;
                }
    }
    return 0;
}

// 1-layer halo map of a level with m cells per block edge. Entries per target
// block, grouped per source leaf in first-appearance order, i-j-k loop order.
// idx[n][8] = tb,ti,tj,tk,sb,i0,j0,k0 of the reference's unclamped
// interpolation; wx[n][6] = weights (3), source-frame centre (3).
// clamped[n] = 1 where the reference's position falls outside [1,m] (the GPU
// clamps those to the source interior; the reference reads a source ghost).
int64_t orc_hc_halo(void* h, int32_t m, int32_t* idx, double* wx, int32_t* clamped, int64_t cap) {
    int32_t nb, ny;
    orc_num_blocks(h, &nb, &ny);
    std::vector<double> rng((size_t)nb * 6);
    std::vector<int32_t> fl(nb);
    orc_block_ranges(h, rng.data());
    orc_block_flags(h, fl.data());
    std::vector<Geo> G(nb);
    for (int b = 0; b < nb; ++b) G[b].init(&rng[(size_t)b * 6], m);
    int64_t n = 0;
    for (int b = 0; b < nb; ++b) {
        // ModGC_FindHC_Single: owner of every ghost of the 1-layer padded block
        std::vector<int32_t> owner((size_t)(m + 2) * (m + 2) * (m + 2), -777);
        auto O = [&](int i, int j, int k) -> int32_t& { return owner[((size_t)i * (m + 2) + j) * (m + 2) + k]; };
        for (int i = 0; i <= m + 1; ++i)
            for (int j = 0; j <= m + 1; ++j)
                for (int k = 0; k <= m + 1; ++k)
                    if (i < 1 || j < 1 || k < 1 || i > m || j > m || k > m) {
                        const double rtp[3] = {G[b].xI[0][i], G[b].xI[1][j], G[b].xI[2][k]};
                        const int leaf = orc_find_leaf(h, rtp, fl[b] & 1);
                        if (leaf >= 0) O(i, j, k) = leaf;
                    }
        // ModGC_GetHC_Targets_single: face ghosts only, grouped per source
        auto face = [&](int i, int j, int k) {
            return ((i == 0 || i == m + 1) ? 1 : 0) + ((j == 0 || j == m + 1) ? 1 : 0) + ((k == 0 || k == m + 1) ? 1 : 0);
        };
        std::vector<int32_t> uniq;
        for (int i = 0; i <= m + 1; ++i)
            for (int j = 0; j <= m + 1; ++j)
                for (int k = 0; k <= m + 1; ++k)
                    if (face(i, j, k) == 1 && O(i, j, k) != -777 &&
                        std::find(uniq.begin(), uniq.end(), O(i, j, k)) == uniq.end())
                        uniq.push_back(O(i, j, k));
        for (int32_t s : uniq)
            for (int i = 0; i <= m + 1; ++i)
                for (int j = 0; j <= m + 1; ++j)
                    for (int k = 0; k <= m + 1; ++k) {
                        if (face(i, j, k) != 1 || O(i, j, k) != s) continue;
                        if (n >= cap) return -1;
                        const double x[3] = {G[b].xI[0][i], G[b].xI[1][j], G[b].xI[2][k]};
                        double xs[3];
                        if ((fl[s] & 1) == (fl[b] & 1)) std::memcpy(xs, x, sizeof x);
                        else orc_coord_conv(x, xs);
                        // ModMath_3D_interpolate_1D with ng=1: posi = 0 + (x-x(0))/(x(2)-x(1)), no clamp
                        int base[3];
                        double w[3];
                        int cl = 0;
                        for (int d = 0; d < 3; ++d) {
                            const std::vector<double>& X = G[s].xI[d];
                            const double pos = (double)((float)(-1) + 1.0f) + (xs[d] - X[0]) / (X[2] - X[1]);
                            base[d] = (int)std::floor(pos);
                            w[d] = pos - base[d];
                            if (pos < 1.0 || pos > (double)m) cl = 1;
                        }
                        if (idx) {
                            const int32_t v[8] = {b, i, j, k, s, base[0], base[1], base[2]};
                            std::memcpy(idx + 8 * n, v, sizeof v);
                            for (int d = 0; d < 3; ++d) { wx[6 * n + d] = w[d]; wx[6 * n + 3 + d] = xs[d]; }
                            clamped[n] = cl;
                        }
                        ++n;
                    }
    }
    return n;
}

// y = A x (3_5/ModLinearSolver.f90:43-50) on level grids with m cells per block
// edge; x is the padded vector [b][m+2][m+2][m+2] (halo already filled).
int orc_spmv(int32_t nb, int32_t m, const double* Aii, const double* Ai, const double* Aj, const double* Ak,
             const double* xp, double* y) {
    const int p = m + 2;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b)
        for (int k = 1; k <= m; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= m; ++i) {
                    auto X = [&](int ii, int jj, int kk) { return xp[(((size_t)b * p + kk) * p + jj) * p + ii]; };
                    y[cidx(m, b, i, j, k)] = Aii[cidx(m, b, i, j, k)] * X(i, j, k) + Ai[fidx_i(m, b, i, j, k)] * X(i - 1, j, k) +
                                             Ai[fidx_i(m, b, i + 1, j, k)] * X(i + 1, j, k) + Aj[fidx_j(m, b, i, j, k)] * X(i, j - 1, k) +
                                             Aj[fidx_j(m, b, i, j + 1, k)] * X(i, j + 1, k) + Ak[fidx_k(m, b, i, j, k)] * X(i, j, k - 1) +
                                             Ak[fidx_k(m, b, i, j, k + 1)] * X(i, j, k + 1);
                }
    return 0;
}

// Fill the 1-layer halo of a padded vector from (idx, w) entries with the
// trilinear form of 3_5/ModMath.f90:238-246; strides of zero-weight directions
// collapse onto the base cell (only the sign of an exact zero can differ).
int orc_halo_fill(int32_t m, const int32_t* idx, const double* w6, int64_t n, double* xp) {
    const int p = m + 2;
    // every entry writes its own ghost cell and reads interior cells only
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; ++e) {
        const int32_t* v = idx + 8 * e;
        const double* w = w6 + 6 * e;
        auto X = [&](int b, int i, int j, int k) { return xp[(((size_t)b * p + k) * p + j) * p + i]; };
        const int s = v[4], i0 = v[5], j0 = v[6], k0 = v[7];
        const int di = w[0] != 0.0, dj = w[1] != 0.0, dk = w[2] != 0.0;
        const double wi = w[0], wj = w[1], wk = w[2];
        const double val = X(s, i0, j0, k0) * (1. - wi) * (1. - wj) * (1. - wk) + X(s, i0 + di, j0, k0) * (wi) * (1. - wj) * (1. - wk) +
                           X(s, i0, j0 + dj, k0) * (1. - wi) * (wj) * (1. - wk) + X(s, i0, j0, k0 + dk) * (1. - wi) * (1. - wj) * (wk) +
                           X(s, i0 + di, j0 + dj, k0) * (wi) * (wj) * (1. - wk) + X(s, i0, j0 + dj, k0 + dk) * (1. - wi) * (wj) * (wk) +
                           X(s, i0 + di, j0, k0 + dk) * (wi) * (1. - wj) * (wk) + X(s, i0 + di, j0 + dj, k0 + dk) * (wi) * (wj) * (wk);
        xp[(((size_t)v[0] * p + v[3]) * p + v[2]) * p + v[1]] = val;
    }
    return 0;
}

// ---- V-cycle components (FP32, the GPU smoother's precision) -----------------
// Restriction: coarse cell (I,J,K) = the sum of its 8 children in the order of
// ModMath_rebin_3D_factor2 (3_6/ModMath.f90:360-367: (1,1,1), (2,1,1), (1,2,1),
// (2,2,1), (1,1,2), (2,1,2), (1,2,2), (2,2,2)), summed left to right, without
// the reference's /8: the operators are volume-integrated, so the coarse
// right-hand side is R = P^T of the fine residual. res, rc interior [b][k][j][i].
int orc_mg_restrict(int32_t nb, int32_t m, const float* res, float* rc) {
    const int mc = m / 2;
    for (int b = 0; b < nb; ++b)
        for (int K = 1; K <= mc; ++K)
            for (int J = 1; J <= mc; ++J)
                for (int I = 1; I <= mc; ++I) {
                    auto F = [&](int i, int j, int k) { return res[cidx(m, b, 2 * I - 2 + i, 2 * J - 2 + j, 2 * K - 2 + k)]; };
                    rc[cidx(mc, b, I, J, K)] =
                        F(1, 1, 1) + F(2, 1, 1) + F(1, 2, 1) + F(2, 2, 1) + F(1, 1, 2) + F(2, 1, 2) + F(1, 2, 2) + F(2, 2, 2);
                }
    return 0;
}

// Prolongation by injection (ModMath_prolongate_3D_factor2, 3_6/ModMath.f90:
// 370-384: each coarse value to its 2x2x2 children), added to the fine
// correction zf (interior [b][k][j][i] of the fine level, m cells per edge).
int orc_mg_prolong_add(int32_t nb, int32_t m, const float* zc, float* zf) {
    const int mc = m / 2;
    for (int b = 0; b < nb; ++b)
        for (int k = 1; k <= m; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= m; ++i)
                    zf[cidx(m, b, i, j, k)] += zc[cidx(mc, b, (i + 1) / 2, (j + 1) / 2, (k + 1) / 2)];
    return 0;
}

// One red-black Gauss-Seidel half sweep: every cell with (i+j+k) % 2 ==
// colour takes the Jacobi update of ModMultigrid_Jacobi_Mz_r
// (3_5/ModMultigrid.f90:316-324), z = (r - Ai z(i-1) - Ai z(i+1) - Aj z(j-1)
// - Aj z(j+1) - Ak z(k-1) - Ak z(k+1)) / Aii, left to right in FP32; its
// neighbours are of the other colour, so the order of cells is immaterial.
// zp padded [b][m+2]^3 with its halo filled.
int orc_mg_rbgs(int32_t nb, int32_t m, const float* Aii, const float* Ai, const float* Aj, const float* Ak,
                const float* r, float* zp, int32_t colour) {
    const int p = m + 2;
    for (int b = 0; b < nb; ++b)
        for (int k = 1; k <= m; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= m; ++i) {
                    if (((i + j + k) & 1) != colour) continue;
                    auto Z = [&](int ii, int jj, int kk) -> float& { return zp[(((size_t)b * p + kk) * p + jj) * p + ii]; };
                    float v = r[cidx(m, b, i, j, k)] - Ai[fidx_i(m, b, i, j, k)] * Z(i - 1, j, k);
                    v = v - Ai[fidx_i(m, b, i + 1, j, k)] * Z(i + 1, j, k);
                    v = v - Aj[fidx_j(m, b, i, j, k)] * Z(i, j - 1, k);
                    v = v - Aj[fidx_j(m, b, i, j + 1, k)] * Z(i, j + 1, k);
                    v = v - Ak[fidx_k(m, b, i, j, k)] * Z(i, j, k - 1);
                    v = v - Ak[fidx_k(m, b, i, j, k + 1)] * Z(i, j, k + 1);
                    Z(i, j, k) = v / Aii[cidx(m, b, i, j, k)];
                }
    return 0;
}

}  // extern "C"

// ---- CPU reference solve (FP64) ---------------------------------------------
namespace {

struct MgLevel {
    int m = 0;
    const double *Aii, *Ai, *Aj, *Ak;
    const int32_t* idx;   // halo [n][8]
    const double* w6;     // halo [n][6]
    int64_t nh;
    std::vector<double> z, r, res;   // z padded; r, res interior
};

struct MgSolver {
    int nb, np, nl, nu_pre, nu_post, nu_coarse;
    const int32_t* bprob;
    std::vector<MgLevel> L;

    size_t nint(int l) const { return (size_t)nb * L[l].m * L[l].m * L[l].m; }
    size_t npad(int l) const { const size_t p = L[l].m + 2; return (size_t)nb * p * p * p; }
    void halo(int l, double* xp) const { orc_halo_fill(L[l].m, L[l].idx, L[l].w6, L[l].nh, xp); }
    double& P(int l, std::vector<double>& v, int b, int i, int j, int k) const {
        const size_t p = L[l].m + 2;
        return v[(((size_t)b * p + k) * p + j) * p + i];
    }
    // one red-black half sweep on level l, FP64
    void sweep(int l, int colour) {
        MgLevel& Q = L[l];
        const int m = Q.m, p = m + 2;
        halo(l, Q.z.data());
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b)
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j)
                    for (int i = 1; i <= m; ++i) {
                        if (((i + j + k) & 1) != colour) continue;
                        auto Z = [&](int ii, int jj, int kk) -> double& { return Q.z[(((size_t)b * p + kk) * p + jj) * p + ii]; };
                        double v = Q.r[cidx(m, b, i, j, k)] - Q.Ai[fidx_i(m, b, i, j, k)] * Z(i - 1, j, k);
                        v = v - Q.Ai[fidx_i(m, b, i + 1, j, k)] * Z(i + 1, j, k);
                        v = v - Q.Aj[fidx_j(m, b, i, j, k)] * Z(i, j - 1, k);
                        v = v - Q.Aj[fidx_j(m, b, i, j + 1, k)] * Z(i, j + 1, k);
                        v = v - Q.Ak[fidx_k(m, b, i, j, k)] * Z(i, j, k - 1);
                        v = v - Q.Ak[fidx_k(m, b, i, j, k + 1)] * Z(i, j, k + 1);
                        Z(i, j, k) = v / Q.Aii[cidx(m, b, i, j, k)];
                    }
    }
    // z_0 = M r_0 (L[0].r): V-cycle with the GPU's structure and sweep counts
    void vcycle() {
        for (int l = 0; l < nl; ++l) {
            MgLevel& Q = L[l];
            std::fill(Q.z.begin(), Q.z.end(), 0.0);
            const int sw = (l == nl - 1 && nl > 1) ? nu_coarse : nu_pre;
            for (int s = 0; s < sw; ++s) { sweep(l, 0); sweep(l, 1); }
            if (l + 1 < nl) {
                halo(l, Q.z.data());
                orc_spmv(nb, Q.m, Q.Aii, Q.Ai, Q.Aj, Q.Ak, Q.z.data(), Q.res.data());
                for (size_t c = 0; c < Q.res.size(); ++c) Q.res[c] = Q.r[c] - Q.res[c];
                MgLevel& C = L[l + 1];
                const int m = Q.m, mc = C.m;
#pragma omp parallel for schedule(static)
                for (int b = 0; b < nb; ++b)
                    for (int K = 1; K <= mc; ++K)
                        for (int J = 1; J <= mc; ++J)
                            for (int I = 1; I <= mc; ++I) {
                                auto F = [&](int i, int j, int k) {
                                    return Q.res[cidx(m, b, 2 * I - 2 + i, 2 * J - 2 + j, 2 * K - 2 + k)];
                                };
                                C.r[cidx(mc, b, I, J, K)] = F(1, 1, 1) + F(2, 1, 1) + F(1, 2, 1) + F(2, 2, 1) + F(1, 1, 2) +
                                                            F(2, 1, 2) + F(1, 2, 2) + F(2, 2, 2);
                            }
            }
        }
        for (int l = nl - 2; l >= 0; --l) {
            MgLevel& Q = L[l];
            MgLevel& C = L[l + 1];
            const int m = Q.m;
#pragma omp parallel for schedule(static)
            for (int b = 0; b < nb; ++b)
                for (int k = 1; k <= m; ++k)
                    for (int j = 1; j <= m; ++j)
                        for (int i = 1; i <= m; ++i) P(l, Q.z, b, i, j, k) += P(l + 1, C.z, b, (i + 1) / 2, (j + 1) / 2, (k + 1) / 2);
            for (int s = 0; s < nu_post; ++s) { sweep(l, 1); sweep(l, 0); }
        }
    }
};

}  // namespace

extern "C" {

// CPU FP64 MG-preconditioned flexible CG of a batch of problems (blocks of
// problem q share its scalars), the GPU solve's algorithm entirely in FP64:
// the same Galerkin levels, halo maps and red-black V-cycle. ops: per level
// Aii, Ai, Aj, Ak (4 pointers per level); halo: per level idx [n][8] and w6
// [n][6] with counts nh[l]; m0 cells per block edge at level 0. x (interior
// [b][m0^3]) holds the initial guess and receives the solution; each problem
// iterates until its true FP64 relative residual is <= tol (checked every
// iteration on a recomputed b - A x) or max_iter. rel[np] receives the final
// relative residuals; returns the iterations taken.
int orc_mg_solve(int32_t nb, int32_t np, const int32_t* bprob, int32_t nl, int32_t m0, const double* const* ops,
                 const int32_t* const* hidx, const double* const* hw6, const int64_t* nh, int32_t nu_pre, int32_t nu_post,
                 int32_t nu_coarse, const double* bvec, double* x, double tol, int32_t max_iter, double* rel) {
    MgSolver S;
    S.nb = nb; S.np = np; S.nl = nl; S.bprob = bprob;
    S.nu_pre = nu_pre; S.nu_post = nu_post; S.nu_coarse = nu_coarse;
    S.L.resize(nl);
    for (int l = 0; l < nl; ++l) {
        MgLevel& Q = S.L[l];
        Q.m = m0 >> l;
        Q.Aii = ops[4 * l]; Q.Ai = ops[4 * l + 1]; Q.Aj = ops[4 * l + 2]; Q.Ak = ops[4 * l + 3];
        Q.idx = hidx[l]; Q.w6 = hw6[l]; Q.nh = nh[l];
        Q.z.assign(S.npad(l), 0.0);
        Q.r.assign(S.nint(l), 0.0);
        Q.res.assign(S.nint(l), 0.0);
    }
    const int m = m0;
    const size_t per = (size_t)m * m * m, n = (size_t)nb * per;
    MgLevel& Z = S.L[0];
    std::vector<double> xp(S.npad(0), 0.0), pp(S.npad(0), 0.0), r(n), z(n), Ap(n);
    auto scatter = [&](const std::vector<double>& v, std::vector<double>& vp, const double* src) {
        (void)v;
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b)
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j)
                    for (int i = 1; i <= m; ++i) S.P(0, vp, b, i, j, k) = src[cidx(m, b, i, j, k)];
    };
    std::vector<double> part(nb);
    auto dots = [&](const double* a, const double* b2, std::vector<double>& out) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b) {
            double s = 0;
            for (size_t c = 0; c < per; ++c) s += a[(size_t)b * per + c] * b2[(size_t)b * per + c];
            part[b] = s;
        }
        std::fill(out.begin(), out.end(), 0.0);
        for (int b = 0; b < nb; ++b) out[bprob[b]] += part[b];
    };
    std::vector<double> bb(np), rr(np), pAp(np), pr(np), zAp(np);
    dots(bvec, bvec, bb);
    for (auto& v : bb) if (!(v > 0)) v = 1.0;
    auto true_residual = [&]() {
        scatter(r, xp, x);
        S.halo(0, xp.data());
        orc_spmv(nb, m, Z.Aii, Z.Ai, Z.Aj, Z.Ak, xp.data(), r.data());
        for (size_t c = 0; c < n; ++c) r[c] = bvec[c] - r[c];
        dots(r.data(), r.data(), rr);
    };
    std::vector<int> active(np, 1);
    auto check = [&]() {
        bool any = false;
        for (int q = 0; q < np; ++q) {
            rel[q] = std::sqrt(rr[q] / bb[q]);
            active[q] = rel[q] > tol;
            any = any || active[q];
        }
        return any;
    };
    auto precondition = [&]() {
        std::copy(r.begin(), r.end(), Z.r.begin());
        S.vcycle();
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b)
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j)
                    for (int i = 1; i <= m; ++i) z[cidx(m, b, i, j, k)] = S.P(0, Z.z, b, i, j, k);
    };
    true_residual();
    if (!check()) return 0;
    precondition();
    scatter(z, pp, z.data());
    int it = 0;
    while (it < max_iter) {
        ++it;
        S.halo(0, pp.data());
        orc_spmv(nb, m, Z.Aii, Z.Ai, Z.Aj, Z.Ak, pp.data(), Ap.data());
        std::vector<double> pint(n);
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b)
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j)
                    for (int i = 1; i <= m; ++i) pint[cidx(m, b, i, j, k)] = S.P(0, pp, b, i, j, k);
        dots(pint.data(), Ap.data(), pAp);
        dots(pint.data(), r.data(), pr);
        for (int b = 0; b < nb; ++b) {
            const int q = bprob[b];
            const double al = (active[q] && pAp[q] != 0.0) ? pr[q] / pAp[q] : 0.0;
            for (size_t c = 0; c < per; ++c) x[(size_t)b * per + c] += al * pint[(size_t)b * per + c];
        }
        true_residual();
        if (!check()) break;
        precondition();
        dots(z.data(), Ap.data(), zAp);
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b) {
            const int q = bprob[b];
            if (!active[q]) continue;
            const double be = pAp[q] != 0.0 ? -zAp[q] / pAp[q] : 0.0;
            for (int k = 1; k <= m; ++k)
                for (int j = 1; j <= m; ++j)
                    for (int i = 1; i <= m; ++i) {
                        double& pv = S.P(0, pp, b, i, j, k);
                        pv = z[cidx(m, b, i, j, k)] + be * pv;
                    }
        }
    }
    return it;
}

}  // extern "C"
