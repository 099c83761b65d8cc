// solver_host.cpp -- multigrid levels, 1-layer halo maps and operator assembly.
//
// Default-real literals of the 3_5 Fortran are reproduced as FP32 constants;
// the arithmetic itself is FP64 (the reference's solver runs in FP32; this is
// the FP64 form the GPU solver is built on).
#include "solver.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>

namespace falcon {

static const double kRsun = (double)6.955e10f;

static inline void yy_convert2(const double* a, double* b) {
    const double st = std::sin(a[1]), ct = std::cos(a[1]);
    const double sp = std::sin(a[2]), cp = std::cos(a[2]);
    b[0] = a[0];
    b[1] = std::acos(st * sp);
    const double den = std::sqrt(st * st * (cp * cp) + ct * ct);
    b[2] = std::copysign(std::fabs(std::acos(-(st * cp) / den)), ct);
}

// ---- level geometry (3_5/ModMultigrid.f90:97-233) -------------------------
void LevelGeometry::init(const double r[3][2], const int mm[3]) {
    for (int d = 0; d < 3; ++d) m[d] = mm[d];
    std::vector<double>* C[3] = {&xiI, &xjI, &xkI};
    std::vector<double>* F[3] = {&xiF, &xjF, &xkF};
    for (int d = 0; d < 3; ++d) {
        const int n = m[d];
        C[d]->resize(n + 2);
        F[d]->resize(n + 2);
        for (int i = 0; i <= n + 1; ++i)
            (*C[d])[i] = (r[d][0] * (double)((float)(n - i) + 0.5f) + r[d][1] * (double)((float)i - 0.5f)) / n;
        for (int i = 1; i <= n + 1; ++i) (*F[d])[i] = (r[d][0] * (double)(n + 1 - i) + r[d][1] * (double)(i - 1)) / n;
    }
    dxi = (r[0][1] - r[0][0]) / m[0];
    dxj = (r[1][1] - r[1][0]) / m[1];
    dxk = (r[2][1] - r[2][0]) / m[2];
}
double LevelGeometry::Si(int i, int j, int k) const {
    return xiF[i] * xiF[i] * (std::cos(xjF[j]) - std::cos(xjF[j + 1])) * (xkF[k + 1] - xkF[k]);
}
double LevelGeometry::Sj(int i, int j, int k) const {
    return 0.5 * (xiF[i + 1] * xiF[i + 1] - xiF[i] * xiF[i]) * (xkF[k + 1] - xkF[k]) * std::sin(xjF[j]);
}
double LevelGeometry::Sk(int i, int j, int k) const {
    (void)k;
    return 0.5 * (xiF[i + 1] * xiF[i + 1] - xiF[i] * xiF[i]) * (xjF[j + 1] - xjF[j]);
}
double LevelGeometry::Di(int, int, int) const { return dxi; }
double LevelGeometry::Dj(int i, int, int) const { return xiI[i] * dxj; }
double LevelGeometry::Dk(int i, int j, int) const { return xiI[i] * dxk * std::sin(xjI[j]); }
double LevelGeometry::Vol(int i, int j, int k) const {
    return (double)(1.0f / 3.0f) * (xiF[i + 1] * xiF[i + 1] * xiF[i + 1] - xiF[i] * xiF[i] * xiF[i]) *
           (std::cos(xjF[j]) - std::cos(xjF[j + 1])) * (xkF[k + 1] - xkF[k]);
}

// ---- levels and halo maps ---------------------------------------------------
std::string build_solver_levels(SolverProblemSet& S, const std::vector<falcon_config>& cfgs, int nlevels_max) {
    S.nproblems = (int)cfgs.size();
    S.grids.assign(S.nproblems, Grid());
    S.problem_first_block.assign(S.nproblems + 1, 0);
    int n0[3] = {0, 0, 0};
    for (int p = 0; p < S.nproblems; ++p) {
        std::string e = S.grids[p].build(cfgs[p], false);
        if (!e.empty()) return e;
        const Grid& g = S.grids[p];
        if (p == 0) { n0[0] = g.ni; n0[1] = g.nj; n0[2] = g.nk; }
        if (g.ni != n0[0] || g.nj != n0[1] || g.nk != n0[2]) return "all problems of a batch must share the block size";
        S.problem_first_block[p + 1] = S.problem_first_block[p] + g.nblocks;
    }
    S.nblocks = S.problem_first_block[S.nproblems];
    if ((int64_t)S.nblocks * (n0[0] + 2) * (n0[1] + 2) * (n0[2] + 2) >= (int64_t)INT32_MAX)
        return "solver grid too large for 32-bit offsets";
    // levels: largest power-of-two divisor depth (3_5/ModMultigrid.f90:76-88)
    int nl = 0;
    for (int l = 1; l <= nlevels_max; ++l) {
        const int f = 1 << (l - 1);
        if (n0[0] % f == 0 && n0[1] % f == 0 && n0[2] % f == 0 && n0[0] / f >= 2 && n0[1] / f >= 2 && n0[2] / f >= 2)
            nl = l;
        else
            break;
    }
    S.nlevels = nl;
    S.block_problem.resize(S.nblocks);
    S.block_flags.resize(S.nblocks);
    for (int p = 0; p < S.nproblems; ++p)
        for (int b = 0; b < S.grids[p].nblocks; ++b) {
            S.block_problem[S.problem_first_block[p] + b] = p;
            S.block_flags[S.problem_first_block[p] + b] = S.grids[p].flags[b];
        }
    S.L.assign(nl, SolverLevel());
    for (int l = 0; l < nl; ++l) {
        SolverLevel& L = S.L[l];
        for (int d = 0; d < 3; ++d) L.m[d] = n0[d] >> l;
        const int mi = L.m[0], mj = L.m[1], mk = L.m[2];
        L.xi.assign((size_t)S.nblocks * (mi + 2), 0.0);
        L.xj.assign((size_t)S.nblocks * (mj + 2), 0.0);
        L.xk.assign((size_t)S.nblocks * (mk + 2), 0.0);
        L.dx.assign((size_t)S.nblocks * 3, 0.0);
        std::vector<std::vector<HaloEntry>> per(S.nblocks);
#pragma omp parallel for schedule(dynamic, 4)
        for (int gb = 0; gb < S.nblocks; ++gb) {
            const int p = S.block_problem[gb];
            const Grid& g = S.grids[p];
            const int b = gb - S.problem_first_block[p];
            double rng[3][2];
            std::memcpy(rng, &g.ranges[(size_t)b * 6], sizeof(rng));
            LevelGeometry G;
            G.init(rng, L.m);
            std::copy(G.xiI.begin(), G.xiI.end(), L.xi.begin() + (size_t)gb * (mi + 2));
            std::copy(G.xjI.begin(), G.xjI.end(), L.xj.begin() + (size_t)gb * (mj + 2));
            std::copy(G.xkI.begin(), G.xkI.end(), L.xk.begin() + (size_t)gb * (mk + 2));
            L.dx[3 * gb] = G.dxi; L.dx[3 * gb + 1] = G.dxj; L.dx[3 * gb + 2] = G.dxk;
        }
        // halo: face ghosts only (exactly one index outside, 3_5/ModGC.f90:210-214)
#pragma omp parallel for schedule(dynamic, 4)
        for (int gb = 0; gb < S.nblocks; ++gb) {
            const int p = S.block_problem[gb];
            const Grid& g = S.grids[p];
            const int off = S.problem_first_block[p];
            const bool yin = g.flags[gb - off] & 1;
            const double* X = &L.xi[(size_t)gb * (mi + 2)];
            const double* Y = &L.xj[(size_t)gb * (mj + 2)];
            const double* Z = &L.xk[(size_t)gb * (mk + 2)];
            for (int i = 0; i <= mi + 1; ++i)
                for (int j = 0; j <= mj + 1; ++j)
                    for (int k = 0; k <= mk + 1; ++k) {
                        const int out = (i == 0 || i == mi + 1) + (j == 0 || j == mj + 1) + (k == 0 || k == mk + 1);
                        if (out != 1) continue;
                        const double rtp[3] = {X[i], Y[j], Z[k]};
                        const int own = g.find_leaf(rtp, yin);
                        if (own < 0) continue;   // radial physical boundary
                        HaloEntry h{};
                        h.tb = gb; h.ti = i; h.tj = j; h.tk = k;
                        h.sb = off + own;
                        const bool syin = g.flags[own] & 1;
                        if (syin == yin) std::memcpy(h.src_x, rtp, sizeof(rtp));
                        else yy_convert2(rtp, h.src_x);
                        const double* SX[3] = {&L.xi[(size_t)h.sb * (mi + 2)], &L.xj[(size_t)h.sb * (mj + 2)],
                                               &L.xk[(size_t)h.sb * (mk + 2)]};
                        int base[3];
                        for (int d = 0; d < 3; ++d) {
                            // posi = (x - x(0))/(x(2)-x(1)) (ng=1), clamped to the source interior
                            const double dd = SX[d][2] - SX[d][1];
                            double pos = (h.src_x[d] - SX[d][0]) / dd;
                            pos = std::max(std::min(pos, (double)L.m[d]), 1.0);
                            base[d] = (int)std::floor(pos);
                            h.w[d] = pos - base[d];
                            if (base[d] == L.m[d]) h.w[d] = 0.0;
                        }
                        h.i0 = base[0]; h.j0 = base[1]; h.k0 = base[2];
                        per[gb].push_back(h);
                    }
        }
        L.halo.clear();
        for (auto& v : per) L.halo.insert(L.halo.end(), v.begin(), v.end());
    }
    return "";
}

// ---- PFSS operator (3_5/ModPFSS.f90:21-100) ---------------------------------
void assemble_pfss(SolverProblemSet& S, const std::vector<double>& br_bottom) {
    for (int l = 0; l < 1; ++l) {
        SolverLevel& L = S.L[l];
        const int mi = L.m[0], mj = L.m[1], mk = L.m[2];
        const size_t ni_ = (size_t)mi * mj * mk;
        L.Aii.assign((size_t)S.nblocks * ni_, 0.0);
        L.Ai.assign((size_t)S.nblocks * (mi + 1) * mj * mk, 0.0);
        L.Aj.assign((size_t)S.nblocks * mi * (mj + 1) * mk, 0.0);
        L.Ak.assign((size_t)S.nblocks * mi * mj * (mk + 1), 0.0);
        L.V.assign((size_t)S.nblocks * ni_, 0.0);
#pragma omp parallel for schedule(static)
        for (int gb = 0; gb < S.nblocks; ++gb) {
            const int p = S.block_problem[gb];
            const Grid& g = S.grids[p];
            const int b = gb - S.problem_first_block[p];
            double rng[3][2];
            std::memcpy(rng, &g.ranges[(size_t)b * 6], sizeof(rng));
            LevelGeometry G;
            G.init(rng, L.m);
            double* Ai = &L.Ai[(size_t)gb * (mi + 1) * mj * mk];
            double* Aj = &L.Aj[(size_t)gb * mi * (mj + 1) * mk];
            double* Ak = &L.Ak[(size_t)gb * mi * mj * (mk + 1)];
            double* Aii = &L.Aii[(size_t)gb * ni_];
            double* V = &L.V[(size_t)gb * ni_];
            auto ai = [&](int i, int j, int k) -> double& { return Ai[((size_t)(k - 1) * mj + (j - 1)) * (mi + 1) + (i - 1)]; };
            auto aj = [&](int i, int j, int k) -> double& { return Aj[((size_t)(k - 1) * (mj + 1) + (j - 1)) * mi + (i - 1)]; };
            auto ak = [&](int i, int j, int k) -> double& { return Ak[((size_t)(k - 1) * mj + (j - 1)) * mi + (i - 1)]; };
            for (int k = 1; k <= mk; ++k)
                for (int j = 1; j <= mj; ++j)
                    for (int i = 1; i <= mi + 1; ++i) ai(i, j, k) = -G.Si(i, j, k) / G.Di(i, j, k);
            for (int k = 1; k <= mk; ++k)
                for (int j = 1; j <= mj + 1; ++j)
                    for (int i = 1; i <= mi; ++i) aj(i, j, k) = -G.Sj(i, j, k) / G.Dj(i, j, k);
            for (int k = 1; k <= mk + 1; ++k)
                for (int j = 1; j <= mj; ++j)
                    for (int i = 1; i <= mi; ++i) ak(i, j, k) = -G.Sk(i, j, k) / G.Dk(i, j, k);
            const bool top = g.flags[b] & 2, bottom = g.flags[b] & 4;
            if (bottom)
                for (int k = 1; k <= mk; ++k)
                    for (int j = 1; j <= mj; ++j) ai(1, j, k) = 0.0;
            for (int k = 1; k <= mk; ++k)
                for (int j = 1; j <= mj; ++j)
                    for (int i = 1; i <= mi; ++i) {
                        const size_t c = ((size_t)(k - 1) * mj + (j - 1)) * mi + (i - 1);
                        Aii[c] = -(ai(i, j, k) + ai(i + 1, j, k) + aj(i, j, k) + aj(i, j + 1, k) + ak(i, j, k) +
                                   ak(i, j, k + 1));
                        V[c] = G.Vol(i, j, k);
                    }
            if (top)
                for (int k = 1; k <= mk; ++k)
                    for (int j = 1; j <= mj; ++j) {
                        const size_t c = ((size_t)(k - 1) * mj + (j - 1)) * mi + (mi - 1);
                        Aii[c] = Aii[c] - ai(mi + 1, j, k);
                        ai(mi + 1, j, k) = 0.0;
                    }
        }
    }
    pfss_rhs(S, br_bottom);
    S.x0.assign(S.b.size(), 0.0);
}

// right-hand side: b(1,:,:) = Br * Si(1,:,:) on bottom blocks, 0 elsewhere
// (3_5/ModPFSS.f90:45-48, level 1); keeps Br in S.br
void pfss_rhs(SolverProblemSet& S, const std::vector<double>& br_bottom) {
    SolverLevel& L = S.L[0];
    const int mi = L.m[0], mj = L.m[1], mk = L.m[2];
    S.br.assign((size_t)S.nblocks * mk * mj, 0.0);
    S.b.assign((size_t)S.nblocks * mi * mj * mk, 0.0);
    for (int gb = 0; gb < S.nblocks; ++gb) {
        if (!(S.block_flags[gb] & 4)) continue;
        const int p = S.block_problem[gb];
        const Grid& g = S.grids[p];
        const int b = gb - S.problem_first_block[p];
        double rng[3][2];
        std::memcpy(rng, &g.ranges[(size_t)b * 6], sizeof(rng));
        LevelGeometry G;
        G.init(rng, L.m);
        for (int k = 1; k <= mk; ++k)
            for (int j = 1; j <= mj; ++j) {
                const size_t f = ((size_t)gb * mk + (k - 1)) * mj + (j - 1);
                S.br[f] = br_bottom[f];
                S.b[(size_t)gb * mi * mj * mk + ((size_t)(k - 1) * mj + (j - 1)) * mi] = br_bottom[f] * G.Si(1, j, k);
            }
    }
}

// ---- Galerkin coarsening A_c = P^T A P (P: injection of each coarse value to
// its 8 children) ---------------------------------------------------------------
void galerkin_coarsen(SolverProblemSet& S) {
    for (int l = 1; l < S.nlevels; ++l) {
        const SolverLevel& F = S.L[l - 1];
        SolverLevel& C = S.L[l];
        const int fi = F.m[0], fj = F.m[1], fk = F.m[2];
        const int ci = C.m[0], cj = C.m[1], ck = C.m[2];
        const size_t nF = (size_t)fi * fj * fk, nC = (size_t)ci * cj * ck;
        C.Aii.assign((size_t)S.nblocks * nC, 0.0);
        C.Ai.assign((size_t)S.nblocks * (ci + 1) * cj * ck, 0.0);
        C.Aj.assign((size_t)S.nblocks * ci * (cj + 1) * ck, 0.0);
        C.Ak.assign((size_t)S.nblocks * ci * cj * (ck + 1), 0.0);
        C.V.assign((size_t)S.nblocks * nC, 0.0);
#pragma omp parallel for schedule(static)
        for (int b = 0; b < S.nblocks; ++b) {
            const double* fA = &F.Aii[(size_t)b * nF];
            const double* fI = &F.Ai[(size_t)b * (fi + 1) * fj * fk];
            const double* fJ = &F.Aj[(size_t)b * fi * (fj + 1) * fk];
            const double* fK = &F.Ak[(size_t)b * fi * fj * (fk + 1)];
            const double* fV = &F.V[(size_t)b * nF];
            auto FI = [&](int i, int j, int k) { return fI[((size_t)k * fj + j) * (fi + 1) + i]; };   // 0-based, face i
            auto FJ = [&](int i, int j, int k) { return fJ[((size_t)k * (fj + 1) + j) * fi + i]; };
            auto FK = [&](int i, int j, int k) { return fK[((size_t)k * fj + j) * fi + i]; };
            double* cA = &C.Aii[(size_t)b * nC];
            double* cI = &C.Ai[(size_t)b * (ci + 1) * cj * ck];
            double* cJ = &C.Aj[(size_t)b * ci * (cj + 1) * ck];
            double* cK = &C.Ak[(size_t)b * ci * cj * (ck + 1)];
            double* cV = &C.V[(size_t)b * nC];
            for (int K = 0; K < ck; ++K)
                for (int J = 0; J < cj; ++J)
                    for (int I = 0; I < ci; ++I) {
                        double d = 0.0, v = 0.0;
                        for (int c = 0; c < 8; ++c) {
                            const int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + (c >> 2);
                            d += fA[((size_t)k * fj + j) * fi + i];
                            v += fV[((size_t)k * fj + j) * fi + i];
                        }
                        // internal faces couple two children of the same coarse cell: counted twice
                        for (int a = 0; a < 2; ++a)
                            for (int q = 0; q < 2; ++q) {
                                d += 2.0 * FI(2 * I + 1, 2 * J + a, 2 * K + q);
                                d += 2.0 * FJ(2 * I + a, 2 * J + 1, 2 * K + q);
                                d += 2.0 * FK(2 * I + a, 2 * J + q, 2 * K + 1);
                            }
                        cA[((size_t)K * cj + J) * ci + I] = d;
                        cV[((size_t)K * cj + J) * ci + I] = v;
                    }
            for (int K = 0; K < ck; ++K)
                for (int J = 0; J < cj; ++J)
                    for (int I = 0; I <= ci; ++I) {
                        double s = 0.0;
                        for (int a = 0; a < 2; ++a)
                            for (int q = 0; q < 2; ++q) s += FI(2 * I, 2 * J + a, 2 * K + q);
                        cI[((size_t)K * cj + J) * (ci + 1) + I] = s;
                    }
            for (int K = 0; K < ck; ++K)
                for (int J = 0; J <= cj; ++J)
                    for (int I = 0; I < ci; ++I) {
                        double s = 0.0;
                        for (int a = 0; a < 2; ++a)
                            for (int q = 0; q < 2; ++q) s += FJ(2 * I + a, 2 * J, 2 * K + q);
                        cJ[((size_t)K * (cj + 1) + J) * ci + I] = s;
                    }
            for (int K = 0; K <= ck; ++K)
                for (int J = 0; J < cj; ++J)
                    for (int I = 0; I < ci; ++I) {
                        double s = 0.0;
                        for (int a = 0; a < 2; ++a)
                            for (int q = 0; q < 2; ++q) s += FK(2 * I + a, 2 * J + q, 2 * K);
                        cK[((size_t)K * cj + J) * ci + I] = s;
                    }
        }
    }
}

// ---- synthetic fields -----------------------------------------------------------
static double unit(std::mt19937_64& r) { return (double)(r() >> 11) * (1.0 / 9007199254740992.0); }
static double gauss(std::mt19937_64& r) {   // Box-Muller
    double u1 = unit(r), u2 = unit(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
}

void ConductionField::init(const Polytrope* b, uint64_t seed, double r_lo) {
    bg = b;
    kappa0 = 1.0e-6;          // Spitzer-like coefficient, CGS
    floor_frac = 1.0e-3;
    ell = 0.05 * kRsun;
    std::mt19937_64 rng(seed);
    const int nm = 64;        // Gaussian random field: sum of random cosines
    kx.resize(nm); ky.resize(nm); kz.resize(nm); ph.resize(nm);
    for (int m = 0; m < nm; ++m) {
        kx[m] = gauss(rng) / ell; ky[m] = gauss(rng) / ell; kz[m] = gauss(rng) / ell;
        ph[m] = 2.0 * 3.14159265358979323846 * unit(rng);
    }
    const int nbp = 20 + (int)(unit(rng) * 181.0);   // 20..200 buried bipoles
    for (int n = 0; n < nbp; ++n) {
        const double rc = (0.60 + 0.09 * unit(rng)) * (r_lo / 0.7);
        const double ct = 2.0 * unit(rng) - 1.0, st = std::sqrt(1.0 - ct * ct), phi = 2.0 * 3.14159265358979323846 * unit(rng);
        const double cx = rc * st * std::cos(phi), cy = rc * st * std::sin(phi), cz = rc * ct;
        double ax = gauss(rng), ay = gauss(rng), az = gauss(rng);
        const double an = std::sqrt(ax * ax + ay * ay + az * az);
        const double sep = (0.02 + 0.03 * unit(rng)) * kRsun * 0.5;
        ax *= sep / an; ay *= sep / an; az *= sep / an;
        const double qq = std::exp(gauss(rng)) * 1e20;
        qx.push_back(cx + ax); qy.push_back(cy + ay); qz.push_back(cz + az); q.push_back(qq);
        qx.push_back(cx - ax); qy.push_back(cy - ay); qz.push_back(cz - az); q.push_back(-qq);
    }
}

double ConductionField::temperature(const double* x, double r) const {
    double o[FALCON_NPROF];
    bg->get_vars(r, o);
    double G = 0.0;
    for (size_t m = 0; m < kx.size(); ++m) G += std::cos(kx[m] * x[0] + ky[m] * x[1] + kz[m] * x[2] + ph[m]);
    G *= std::sqrt(2.0 / (double)kx.size());
    return o[3] * std::exp(0.5 * G - 0.125);
}

void ConductionField::bfield(const double* x, double* B) const {
    B[0] = B[1] = B[2] = 0.0;
    for (size_t n = 0; n < q.size(); ++n) {
        const double dx = x[0] - qx[n], dy = x[1] - qy[n], dz = x[2] - qz[n];
        const double d2 = dx * dx + dy * dy + dz * dz;
        const double f = q[n] / (d2 * std::sqrt(d2));
        B[0] += f * dx; B[1] += f * dy; B[2] += f * dz;
    }
}

// kappa on a face with unit normal e (block frame) at Cartesian point x
static double kappa_dir(const ConductionField& F, const double* xyz, double r, const double* e) {
    const double T = F.temperature(xyz, r);
    double B[3];
    F.bfield(xyz, B);
    const double bn = std::sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    const double bd = bn > 0 ? (B[0] * e[0] + B[1] * e[1] + B[2] * e[2]) / bn : 0.0;
    const double kpar = F.kappa0 * std::pow(T, 2.5);
    return kpar * bd * bd + F.floor_frac * F.kappa0 * std::pow(F.bg->T_b, 2.5);
}

// point in the Yin Cartesian frame and the block-frame unit vectors
static void frame(bool yin, double r, double t, double p, double* xyz, double e[3][3]) {
    double ty = t, py = p;
    if (!yin) { double a[3] = {r, t, p}, c[3]; yy_convert2(a, c); ty = c[1]; py = c[2]; }
    xyz[0] = r * std::sin(ty) * std::cos(py);
    xyz[1] = r * std::sin(ty) * std::sin(py);
    xyz[2] = r * std::cos(ty);
    // unit vectors of the block frame expressed in the block frame's Cartesian axes
    const double st = std::sin(t), ct = std::cos(t), sp = std::sin(p), cp = std::cos(p);
    double er[3] = {st * cp, st * sp, ct}, et[3] = {ct * cp, ct * sp, -st}, ep[3] = {-sp, cp, 0.0};
    if (!yin) {
        // Yang Cartesian (x', y', z') = (-x, z, y) of Yin Cartesian: rotate vectors back to Yin axes
        auto rot = [](const double* v, double* o) { o[0] = -v[0]; o[1] = v[2]; o[2] = v[1]; };
        rot(er, e[0]); rot(et, e[1]); rot(ep, e[2]);
    } else {
        for (int d = 0; d < 3; ++d) { e[0][d] = er[d]; e[1][d] = et[d]; e[2][d] = ep[d]; }
    }
}

void assemble_conduction(SolverProblemSet& S, const ConductionField& F, double dt_factor, double* dt_out) {
    const Polytrope& bg = *F.bg;
    const double cv = 1.5 * bg.R_gas;   // ideal gas, gamma = 5/3
    // explicit limit 0.5*min h^2/max(kappa/(rho cv)) on level 1 cell centres
    double dt_ex = 1e300;
    {
        SolverLevel& L = S.L[0];
        const int mi = L.m[0], mj = L.m[1], mk = L.m[2];
#pragma omp parallel for schedule(dynamic) reduction(min : dt_ex)
        for (int gb = 0; gb < S.nblocks; ++gb) {
            const bool yin = S.block_flags[gb] & 1;
            for (int k = 1; k <= mk; k += 2)
                for (int j = 1; j <= mj; j += 2)
                    for (int i = 1; i <= mi; i += 2) {
                        const double r = L.xi[(size_t)gb * (mi + 2) + i], t = L.xj[(size_t)gb * (mj + 2) + j],
                                     p = L.xk[(size_t)gb * (mk + 2) + k];
                        double xyz[3], e[3][3], o[FALCON_NPROF];
                        frame(yin, r, t, p, xyz, e);
                        bg.get_vars(r, o);
                        double kmax = 0;
                        for (int d = 0; d < 3; ++d) kmax = std::max(kmax, kappa_dir(F, xyz, r, e[d]));
                        const double h = std::min(L.dx[3 * gb], std::min(r * L.dx[3 * gb + 1], r * std::sin(t) * L.dx[3 * gb + 2]));
                        dt_ex = std::min(dt_ex, 0.5 * h * h / (kmax / (o[1] * cv)));
                    }
        }
    }
    const double dt = dt_factor * dt_ex;
    if (dt_out) *dt_out = dt;
    for (int l = 0; l < 1; ++l) {
        SolverLevel& L = S.L[l];
        const int mi = L.m[0], mj = L.m[1], mk = L.m[2];
        const size_t nI = (size_t)mi * mj * mk;
        L.Aii.assign((size_t)S.nblocks * nI, 0.0);
        L.Ai.assign((size_t)S.nblocks * (mi + 1) * mj * mk, 0.0);
        L.Aj.assign((size_t)S.nblocks * mi * (mj + 1) * mk, 0.0);
        L.Ak.assign((size_t)S.nblocks * mi * mj * (mk + 1), 0.0);
        L.V.assign((size_t)S.nblocks * nI, 0.0);
        if (l == 0) { S.b.assign((size_t)S.nblocks * nI, 0.0); S.x0.assign(S.b.size(), 0.0); }
#pragma omp parallel for schedule(dynamic)
        for (int gb = 0; gb < S.nblocks; ++gb) {
            const int p = S.block_problem[gb];
            const Grid& g = S.grids[p];
            const int b = gb - S.problem_first_block[p];
            const bool yin = S.block_flags[gb] & 1, top = S.block_flags[gb] & 2, bottom = S.block_flags[gb] & 4;
            double rng[3][2];
            std::memcpy(rng, &g.ranges[(size_t)b * 6], sizeof(rng));
            LevelGeometry G;
            G.init(rng, L.m);
            // kappa at cell centres incl. the ghost layer (per direction)
            const int pi = mi + 2, pj = mj + 2, pk = mk + 2;
            std::vector<double> kap(3 * (size_t)pi * pj * pk, 0.0), T((size_t)pi * pj * pk), rho((size_t)pi);
            for (int i = 0; i < pi; ++i) { double o[FALCON_NPROF]; bg.get_vars(G.xiI[i], o); rho[i] = o[1]; }
            for (int k = 0; k < pk; ++k)
                for (int j = 0; j < pj; ++j)
                    for (int i = 0; i < pi; ++i) {
                        const int out = (i == 0 || i == mi + 1) + (j == 0 || j == mj + 1) + (k == 0 || k == mk + 1);
                        if (out > 1) continue;
                        double xyz[3], e[3][3];
                        frame(yin, G.xiI[i], G.xjI[j], G.xkI[k], xyz, e);
                        const size_t c = ((size_t)k * pj + j) * pi + i;
                        for (int d = 0; d < 3; ++d) kap[(size_t)d * pi * pj * pk + c] = kappa_dir(F, xyz, G.xiI[i], e[d]);
                        if (out == 0) T[c] = F.temperature(xyz, G.xiI[i]);
                    }
            auto K = [&](int d, int i, int j, int k) { return kap[(size_t)d * pi * pj * pk + ((size_t)k * pj + j) * pi + i]; };
            double* Ai = &L.Ai[(size_t)gb * (mi + 1) * mj * mk];
            double* Aj = &L.Aj[(size_t)gb * mi * (mj + 1) * mk];
            double* Ak = &L.Ak[(size_t)gb * mi * mj * (mk + 1)];
            for (int k = 1; k <= mk; ++k)
                for (int j = 1; j <= mj; ++j)
                    for (int i = 1; i <= mi + 1; ++i) {
                        const double kf = 0.5 * (K(0, i - 1, j, k) + K(0, i, j, k));
                        double a = -kf * G.Si(i, j, k) / G.Di(i, j, k);
                        if ((i == 1 && bottom) || (i == mi + 1 && top)) a = 0.0;   // insulating radial boundaries
                        Ai[((size_t)(k - 1) * mj + (j - 1)) * (mi + 1) + (i - 1)] = a;
                    }
            for (int k = 1; k <= mk; ++k)
                for (int j = 1; j <= mj + 1; ++j)
                    for (int i = 1; i <= mi; ++i) {
                        const double kf = 0.5 * (K(1, i, j - 1, k) + K(1, i, j, k));
                        Aj[((size_t)(k - 1) * (mj + 1) + (j - 1)) * mi + (i - 1)] = -kf * G.Sj(i, j, k) / G.Dj(i, j, k);
                    }
            for (int k = 1; k <= mk + 1; ++k)
                for (int j = 1; j <= mj; ++j)
                    for (int i = 1; i <= mi; ++i) {
                        const double kf = 0.5 * (K(2, i, j, k - 1) + K(2, i, j, k));
                        Ak[((size_t)(k - 1) * mj + (j - 1)) * mi + (i - 1)] = -kf * G.Sk(i, j, k) / G.Dk(i, j, k);
                    }
            for (int k = 1; k <= mk; ++k)
                for (int j = 1; j <= mj; ++j)
                    for (int i = 1; i <= mi; ++i) {
                        const size_t c = ((size_t)(k - 1) * mj + (j - 1)) * mi + (i - 1);
                        const double vol = G.Vol(i, j, k);
                        const double diag = rho[i] * cv * vol / dt;
                        const double off = Ai[((size_t)(k - 1) * mj + (j - 1)) * (mi + 1) + (i - 1)] +
                                           Ai[((size_t)(k - 1) * mj + (j - 1)) * (mi + 1) + i] +
                                           Aj[((size_t)(k - 1) * (mj + 1) + (j - 1)) * mi + (i - 1)] +
                                           Aj[((size_t)(k - 1) * (mj + 1) + j) * mi + (i - 1)] +
                                           Ak[((size_t)(k - 1) * mj + (j - 1)) * mi + (i - 1)] +
                                           Ak[((size_t)k * mj + (j - 1)) * mi + (i - 1)];
                        L.Aii[(size_t)gb * nI + c] = diag - off;
                        L.V[(size_t)gb * nI + c] = vol;
                        if (l == 0) {
                            const double Tc = T[((size_t)k * pj + j) * pi + i];
                            S.b[(size_t)gb * nI + c] = diag * Tc;
                            S.x0[(size_t)gb * nI + c] = Tc;
                        }
                    }
        }
    }
}

// ---- synthetic magnetogram ----------------------------------------------------
void Magnetogram::init(uint64_t seed, double r_surface) {
    std::mt19937_64 rng(seed);
    // Poisson(110) number of bipoles, clipped to 20..200 (Knuth's method on log)
    int n = 0;
    {
        double L = std::exp(-110.0), prod = unit(rng);
        while (prod > L && n < 400) { prod *= unit(rng); ++n; }
    }
    n = std::max(20, std::min(200, n));
    const double depth = 0.02 * r_surface;
    for (int b = 0; b < n; ++b) {
        const double lat = (unit(rng) - 0.5) * 1.2, lon = 2.0 * 3.14159265358979323846 * unit(rng);
        const double tilt = gauss(rng) * 0.3, sep = (0.01 + 0.03 * unit(rng)) * r_surface;
        const double flux = std::exp(0.8 * gauss(rng)) * 1e3 * depth * depth;   // log-normal, G cm^2 scale
        const double th = 0.5 * 3.14159265358979323846 - lat, rc = r_surface - depth;
        const double cx = rc * std::sin(th) * std::cos(lon), cy = rc * std::sin(th) * std::sin(lon), cz = rc * std::cos(th);
        // east-west separation rotated by the tilt in the local tangent plane
        const double ex = -std::sin(lon), ey = std::cos(lon), ez = 0.0;
        const double nx = -std::cos(th) * std::cos(lon), ny = -std::cos(th) * std::sin(lon), nz = std::sin(th);
        const double dx = 0.5 * sep * (std::cos(tilt) * ex + std::sin(tilt) * nx);
        const double dy = 0.5 * sep * (std::cos(tilt) * ey + std::sin(tilt) * ny);
        const double dz = 0.5 * sep * (std::cos(tilt) * ez + std::sin(tilt) * nz);
        px.push_back(cx + dx); py.push_back(cy + dy); pz.push_back(cz + dz); q.push_back(flux);
        px.push_back(cx - dx); py.push_back(cy - dy); pz.push_back(cz - dz); q.push_back(-flux);
    }
}

// Br at (r, theta, phi) (Yin frame): point charges (3_5/ModMagnetogram.f90:43-74
// form) plus a 1 G axial dipole
double Magnetogram::br(double r, double t, double p) const {
    const double x = r * std::sin(t) * std::cos(p), y = r * std::sin(t) * std::sin(p), z = r * std::cos(t);
    double s = 0.0;
    for (size_t n = 0; n < q.size(); ++n) {
        const double dx = x - px[n], dy = y - py[n], dz = z - pz[n];
        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
        s += q[n] * (dx * x + dy * y + dz * z) / r / (d * d * d);
    }
    return s + dipole_g * std::cos(t);
}

}  // namespace falcon
