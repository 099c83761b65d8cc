// solver_oracle.cpp -- CPU restatement of the reference's implicit-solver
// components (TEST INFRASTRUCTURE ONLY: the checker for the GPU solvers).
//
//   level geometry  3_5/ModMultigrid.f90:97-233 (iGeometry = 1)
//   PFSS operator   3_5/ModPFSS.f90:21-100 (level 1)
//   1-layer halo    3_5/ModGC.f90:53-76,174-284 (face ghosts, grouped per source
//                   in first-appearance order, i-j-k loop order) and the
//                   interpolation of 3_5/ModMath.f90:208-248
//   SpMV            3_5/ModLinearSolver.f90:34-51
// The reference solver runs in default real (FP32); this restatement keeps the
// operation order and evaluates in FP64, the precision of the GPU outer solve.
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

}  // extern "C"
