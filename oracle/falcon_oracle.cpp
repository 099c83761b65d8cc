// falcon_oracle.cpp -- CPU restatement of Falcon's per-step hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle: the checker that the
// GB300 path is compared against, and the CPU baseline that bench.py times.
// Nothing in the product (falcon_gb300/) links, loads or calls it.
//
// It restates, in the reference's own operation order, the Fortran of
// xianyu2023umich/Falcon snapshot 3_6 (single MPI rank):
//   tree        3_6/ModYinYangTree.f90:91-505, 3_6/ModAMR.f90:13-99
//   geometry    3_6/ModBlock.f90:115-438
//   ghost map   3_6/ModGC.f90:25-147, 3_6/ModCommunication.f90:22-366
//   exchange    3_6/ModCommunication.f90:655-795, 3_6/ModMath.f90:250-293,
//               3_6/ModYinYang.f90:8-61
//   step        3_6/ModAdvance.f90:18-112, 3_6/ModWaveSpeed.f90:8-27,
//               3_6/ModTimeStep.f90:10-30, 3_6/ModBoundary.f90:10-55,
//               3_6/ModEquation.f90:24-162, 3_6/ModSpherical.f90:26-343,
//               3_6/ModDerivative.f90:5-34, 3_6/ModDiffusion.f90:9-150,
//               3_6/ModLinReconstruct.f90:5-49
// Default-real (FP32) literals and ModConst parameters are reproduced as FP32
// values promoted to FP64, exactly as gfortran evaluates them. Build with
// -ffp-contract=off: the reference is compiled without FMA contraction.
//
// Generalisations (documented, not in the reference):
//   - a root tiling: each panel root is split once into N_r x N_t x N_p
//     children with YinYangTree_Divide's own formula, N not limited to 2;
//   - the background is a polytrope served through the get_vars interface
//     (3_6/ModStratification_new.f90:352-384) instead of the FreeEOS tables;
//   - psi (variable 9) is stored as in the reference's MHD block; with
//     DivB_option=0 its RHS is set to 0 each stage (the reference leaves the
//     previous diffusion pass's value there, which is 0 for a psi that starts
//     at 0, the only psi the GPU accepts with DivB_option=0).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/falcon_gb300.h"

namespace orc {

// ---- 3_6/ModConst.f90:2-13 (default real = FP32) -------------------------
static const float  dpi_f = 3.1415926535f;
static const double R_sun = (double)6.955e10f;
static const double k_B = (double)1.380649e-16f;
static const double m_p = (double)1.67262192369e-24f;
static const double gamma_ideal_gas = (double)(5.0f / 3.0f);

static const int NPROF = FALCON_NPROF;
enum { RHO1 = 0, VR = 1, VT = 2, VP = 3, BR = 4, BT = 5, BP = 6, S1 = 7, PSI = 8 };

// ---- background: polytrope through the get_vars interface ----------------
struct Background {
    double n, contrast, mu;
    int xi_mode;
    double rb, rt, zeta_t, K, rho_b, g_b, p_b, R_gas, T_b, c_top;

    double zeta(double r) const { return 1.0 + K * (1.0 / r - 1.0 / rb); }
    void init(const falcon_background_spec& s, double r_lo, double r_hi) {
        n = s.poly_n; contrast = s.density_contrast; mu = s.mu; xi_mode = s.xi_mode;
        rb = r_lo; rt = r_hi;
        zeta_t = std::pow(contrast, -1.0 / n);
        K = (1.0 - zeta_t) / (1.0 / rb - 1.0 / rt);
        rho_b = std::pow(10.0, -0.6841807359334023);   // 3_6/ModStratification_new.f90:29
        g_b = 54340.03688603464;                       // 3_6/ModStratification_new.f90:30
        p_b = rho_b * g_b * rb * rb / ((n + 1.0) * K);
        R_gas = k_B / (mu * m_p);
        T_b = p_b / (rho_b * R_gas);
        double zt = zeta(rt);
        double rho_t = rho_b * std::pow(zt, n);
        double p_t = p_b * std::pow(zt, n + 1.0);
        c_top = std::sqrt(gamma_ideal_gas * p_t / rho_t);
    }
    // out: g, rho0, p0, T0, gamma1, gamma3, diffusion, cooling, Xi
    void get_vars(double r, double* o) const {
        double z = zeta(r);
        double q = rb / r;
        o[0] = g_b * (q * q);
        o[1] = rho_b * std::pow(z, n);
        o[2] = p_b * std::pow(z, n + 1.0);
        o[3] = T_b * z;
        o[4] = gamma_ideal_gas;
        o[5] = gamma_ideal_gas;
        o[6] = 0.0;
        o[7] = 0.0;
        o[8] = xi_mode ? std::sqrt(o[4] * o[2] / o[1]) / c_top : 1.0;
    }
    // 3_6/ModStratification_new.f90:388-432
    double get_middle_r(const double* rr) const {
        const int nn = 200;
        double dr = (rr[1] - rr[0]) / (double)nn;
        std::vector<double> rho(nn + 1), f(nn + 1), cumul(nn + 1);
        double o[NPROF];
        for (int i = 1; i <= nn + 1; ++i) {
            double r = rr[0] + (i - 1) * dr;
            get_vars(r, o);
            rho[i - 1] = o[1];
        }
        f[0] = std::fabs(rho[1] - rho[0]) / (dr * rho[0]);
        f[nn] = std::fabs(rho[nn] - rho[nn - 1]) / (dr * rho[nn]);
        for (int i = 2; i <= nn; ++i)
            f[i - 1] = std::fabs(rho[i] - rho[i - 2]) / (2.0 * dr * rho[i - 1]);
        cumul[0] = 0.0;
        for (int i = 2; i <= nn + 1; ++i)
            cumul[i - 1] = cumul[i - 2] + 0.5 * (f[i - 1] + f[i - 2]) * dr;
        double half_total = 0.5 * cumul[nn];
        double r_middle = rr[1];
        for (int i = 2; i <= nn + 1; ++i) {
            if (cumul[i - 1] >= half_total) {
                r_middle = (rr[0] + (i - 2) * dr) +
                           (half_total - cumul[i - 2]) / (cumul[i - 1] - cumul[i - 2]) * dr;
                break;
            }
        }
        return r_middle;
    }
};

// ---- 3_6/ModYinYang.f90:8-17 ----------------------------------------------
static inline void coord_conv(const double* in, double* out) {
    double st = std::sin(in[1]), sp = std::sin(in[2]), cp = std::cos(in[2]), ct = std::cos(in[1]);
    out[0] = in[0];
    out[1] = std::acos(st * sp);
    double a = std::acos(-(st * cp) / std::sqrt(st * st * (cp * cp) + ct * ct));
    out[2] = std::copysign(std::fabs(a), ct);
}
// 3_6/ModYinYang.f90:34-46 (vector from the frame of rtp_in to the other frame)
static inline void vec_conv(const double* rtp_in, const double* v, double* o) {
    double ro[3];
    coord_conv(rtp_in, ro);
    double s1 = std::sin(rtp_in[2]), s2 = std::sin(ro[2]);
    double c1 = std::cos(rtp_in[2]), s3 = std::sin(ro[1]);
    o[0] = v[0];
    o[1] = -(s1 * s2 * v[1]) - c1 / s3 * v[2];
    o[2] = -(s1 * s2 * v[2]) + c1 / s3 * v[1];
}

// ---- tree (3_6/ModYinYangTree.f90) ----------------------------------------
struct Node {
    bool leaf = true, yin = true;
    double rng[3][2];
    int leaf_id = 0;
    std::vector<Node> ch;
};

static void divide_general(Node& nd, const int N[3]) {
    // 3_6/ModYinYangTree.f90:210-269 with N_rtp(d) = N[d]
    if (nd.leaf) {
        nd.ch.resize((size_t)N[0] * N[1] * N[2]);
        int ic = 0;
        double (*R)[2] = nd.rng;
        for (int ir = 1; ir <= N[0]; ++ir)
            for (int it = 1; it <= N[1]; ++it)
                for (int ip = 1; ip <= N[2]; ++ip) {
                    Node& c = nd.ch[ic++];
                    c.leaf = true; c.yin = nd.yin;
                    float e1 = ((float)(N[0] - ir) + 1.0f) / (float)N[0];
                    float e2 = ((float)(N[0] - ir) + 0.0f) / (float)N[0];
                    float f1 = ((float)(-ir) + 1.0f) / (float)N[0];
                    float f2 = ((float)(-ir) + 0.0f) / (float)N[0];
                    c.rng[0][0] = std::pow(R[0][0], (double)e1) / std::pow(R[0][1], (double)f1);
                    c.rng[0][1] = std::pow(R[0][0], (double)e2) / std::pow(R[0][1], (double)f2);
                    float a1 = (float)(N[1] - it) + 1.0f, a2 = (float)(N[1] - it) + 0.0f;
                    float b1 = (float)(-it) + 1.0f, b2 = (float)(-it) + 0.0f;
                    c.rng[1][0] = R[1][0] * (double)a1 / (double)N[1] - R[1][1] * (double)b1 / (double)N[1];
                    c.rng[1][1] = R[1][0] * (double)a2 / (double)N[1] - R[1][1] * (double)b2 / (double)N[1];
                    float p1 = (float)(N[2] - ip) + 1.0f, p2 = (float)(N[2] - ip) + 0.0f;
                    float q1 = (float)(-ip) + 1.0f, q2 = (float)(-ip) + 0.0f;
                    c.rng[2][0] = R[2][0] * (double)p1 / (double)N[2] - R[2][1] * (double)q1 / (double)N[2];
                    c.rng[2][1] = R[2][0] * (double)p2 / (double)N[2] - R[2][1] * (double)q2 / (double)N[2];
                }
    }
    nd.leaf = false;
}

static void divide_r(Node& nd, int opt, const Background& bg) {
    // 3_6/ModYinYangTree.f90:158-206
    if (nd.leaf) {
        nd.ch.resize(2);
        for (int ic = 1; ic <= 2; ++ic) {
            double r_middle = 0.0;
            if (opt == 1) r_middle = bg.get_middle_r(nd.rng[0]);
            else if (opt == 2) r_middle = (nd.rng[0][0] + nd.rng[0][1]) * 0.5;
            else if (opt == 3) r_middle = std::sqrt(nd.rng[0][0] * nd.rng[0][1]);
            Node& c = nd.ch[ic - 1];
            std::memcpy(c.rng, nd.rng, sizeof(c.rng));
            if (ic == 1) c.rng[0][1] = r_middle; else c.rng[0][0] = r_middle;
            c.leaf = true; c.yin = nd.yin;
        }
    }
    nd.leaf = false;
}

static void divide_r_branch(Node& nd, int opt, const Background& bg) {
    if (nd.leaf) divide_r(nd, opt, bg);
    else for (auto& c : nd.ch) divide_r_branch(c, opt, bg);
}

// 3_6/ModMath.f90:5-16
static bool lines_intersect(const double* a, const double* b) {
    return (a[0] - b[0]) * (a[0] - b[1]) < 0.0 || (a[1] - b[0]) * (a[1] - b[1]) < 0.0 ||
           (b[0] - a[0]) * (b[0] - a[1]) < 0.0 || (b[1] - a[0]) * (b[1] - a[1]) < 0.0;
}

static void amr_branch(Node& nd, const falcon_tree_spec& sp, int l) {
    // 3_6/ModAMR.f90:65-99
    if (nd.leaf) {
        double rr[2] = {sp.amr_range[l][0][0] * R_sun, sp.amr_range[l][0][1] * R_sun};
        int N[3];
        for (int d = 0; d < 3; ++d) N[d] = sp.amr_divide[l][d] ? 2 : 1;
        if (sp.amr_global[l]) {
            if (lines_intersect(nd.rng[0], rr)) divide_general(nd, N);
        } else if (nd.yin) {
            if (lines_intersect(nd.rng[0], rr) && lines_intersect(nd.rng[1], sp.amr_range[l][1]) &&
                lines_intersect(nd.rng[2], sp.amr_range[l][2]))
                divide_general(nd, N);
        }
    } else {
        for (auto& c : nd.ch) amr_branch(c, sp, l);
    }
}

static void label(Node& nd, int& count, std::vector<Node*>& leaves) {
    if (nd.leaf) { nd.leaf_id = ++count; leaves.push_back(&nd); }
    else for (auto& c : nd.ch) label(c, count, leaves);
}

static bool inside(const Node& nd, const double* rtp, bool yin) {
    // 3_6/ModYinYangTree.f90:424-445
    double h[3];
    if (yin == nd.yin) { h[0] = rtp[0]; h[1] = rtp[1]; h[2] = rtp[2]; }
    else coord_conv(rtp, h);
    return (h[0] - nd.rng[0][0]) * (h[0] - nd.rng[0][1]) <= 0.0 &&
           (h[1] - nd.rng[1][0]) * (h[1] - nd.rng[1][1]) <= 0.0 &&
           (h[2] - nd.rng[2][0]) * (h[2] - nd.rng[2][1]) <= 0.0;
}

static const Node* find_branch(const Node& n0, const double* rtp, bool yin) {
    // 3_6/ModYinYangTree.f90:468-505
    const Node* res = nullptr;
    if (inside(n0, rtp, yin)) {
        if (n0.leaf) res = &n0;
        else
            for (const auto& c : n0.ch) {
                if (inside(c, rtp, yin)) res = find_branch(c, rtp, yin);
                if (res) break;
            }
    }
    return res;
}

struct Tree {
    Node yin, yang;
    int nleaf = 0, nleaf_yin = 0;
    double rr[2];
    std::vector<Node*> leaves;

    const Node* find(const double* rtp, bool y) const {
        // 3_6/ModYinYangTree.f90:449-464
        if (inside(yin, rtp, y)) return find_branch(yin, rtp, y);
        return find_branch(yang, rtp, y);
    }
};

// ---- blocks -----------------------------------------------------------------
struct GCList {
    int other;               // leaf id (1-based) of the other block
    bool other_yin;
    std::vector<int> ijk;    // target-side (i,j,k), Fortran indices
    std::vector<double> x;   // coordinates (target frame for targets, source frame for sources)
};

struct Block {
    int id;  // 1-based leaf id
    bool yin, top = false, bottom = false;
    double rng[3][2];
    double dxi, dxj, dxk;
    std::vector<double> xi, xj, xk;   // padded, index (i+ng-1)
    std::vector<double> h;            // interior
    std::vector<double> prof;         // [NPROF][nip]
    // 1D versions of the 3D replicas of ModBlock_InitSSM (3_6/ModBlock.f90:252-264)
    std::vector<double> gamma1, g3m1, rho0, g_over_rho0, p0_over_rho0, rho0T0, heat, Xi;
    std::vector<double> u, urk, R, p1, vwave;
    std::vector<int> owner;           // padded (-777 outside)
    std::vector<GCList> targets, sources;
};

struct Oracle {
    falcon_config cfg;
    int ni, nj, nk, ng, nip, njp, nkp, ncell, nvar = FALCON_NVAR;
    Background bg;
    Tree tree;
    std::vector<Block> blk;
    double dt = 0.0;
    // a rank of a block-sharded run owns blocks [own_first, own_last): the
    // phases, the time step and the exchange then cover owned blocks only
    // (own_last < 0: every block)
    int own_first = 0, own_last = -1;
    bool owned(int b) const { return own_last < 0 || (b >= own_first && b < own_last); }
    std::string err;

    int idx(int i, int j, int k) const { return (i + ng - 1) + nip * ((j + ng - 1) + njp * (k + ng - 1)); }
    int iidx(int i, int j, int k) const { return (i - 1) + ni * ((j - 1) + nj * (k - 1)); }

    void build();
    void init_grid(Block& b);
    void init_ssm(Block& b);
    void derive_ssm(Block& b);
    void find_gc(Block& b);
    void gc_targets(Block& b);
    void gc_sources();
    void exchange(bool rk);
    // one ghost entry's values from source block S (ModMath_1D3D_interpolate_1D1D
    // and, across the Yin-Yang seam, ModYinYang_VecConv_1D)
    void interp(const Block& S, bool rk, const double* x, bool rotate, double* val) const;
    void boundary(Block& b, std::vector<double>& p);
    void equation(Block& b, const std::vector<double>& p);
    void glm(Block& b, const std::vector<double>& p);
    void powell(Block& b, const std::vector<double>& p);
    void diffusion(Block& b, const std::vector<double>& p);
    void wave_speed(Block& b);
    double timestep();
    void step();
    void phase(int ph);
};

void Oracle::build() {
    const falcon_tree_spec& sp = cfg.tree;
    ni = sp.ni; nj = sp.nj; nk = sp.nk; ng = sp.ng;
    nip = ni + 2 * ng; njp = nj + 2 * ng; nkp = nk + 2 * ng;
    ncell = nip * njp * nkp;
    // r_range = r_range_Rsun * R_sun__CGS (3_6/ModReadParameters.f90:71)
    tree.rr[0] = sp.r_range_rsun[0] * R_sun;
    tree.rr[1] = sp.r_range_rsun[1] * R_sun;
    bg.init(cfg.bg, tree.rr[0], tree.rr[1]);
    // YinYangTree_InitTree (3_6/ModYinYangTree.f90:91-110)
    for (Node* root : {&tree.yin, &tree.yang}) {
        root->leaf = true;
        root->yin = (root == &tree.yin);
        root->rng[0][0] = tree.rr[0]; root->rng[0][1] = tree.rr[1];
        root->rng[1][0] = (double)(dpi_f * 0.25f); root->rng[1][1] = (double)(dpi_f * 0.75f);
        root->rng[2][0] = (double)(-(dpi_f * 0.75f)); root->rng[2][1] = (double)(dpi_f * 0.75f);
    }
    // root tiling (generalisation)
    if (sp.root_tiles[0] * sp.root_tiles[1] * sp.root_tiles[2] > 1) {
        divide_general(tree.yin, sp.root_tiles);
        divide_general(tree.yang, sp.root_tiles);
    }
    // ModAMR_set_grid (3_6/ModAMR.f90:13-62)
    for (int l = 0; l < sp.radial_levels; ++l) {
        divide_r_branch(tree.yin, sp.radial_option, bg);
        divide_r_branch(tree.yang, sp.radial_option, bg);
    }
    for (int l = 0; l < sp.n_amr; ++l) {
        amr_branch(tree.yin, sp, l);
        amr_branch(tree.yang, sp, l);
    }
    // YinYangTree_SetAll (3_6/ModYinYangTree.f90:294-344)
    label(tree.yin, tree.nleaf, tree.leaves);
    tree.nleaf_yin = tree.nleaf;
    label(tree.yang, tree.nleaf, tree.leaves);
    blk.resize(tree.nleaf);
    for (int b = 0; b < tree.nleaf; ++b) {
        Block& B = blk[b];
        B.id = b + 1;
        B.yin = B.id <= tree.nleaf_yin;
        std::memcpy(B.rng, tree.leaves[b]->rng, sizeof(B.rng));
        init_grid(B);
        B.u.assign((size_t)nvar * ncell, 0.0);
        B.urk.assign((size_t)nvar * ncell, 0.0);
        B.R.assign((size_t)nvar * ni * nj * nk, 0.0);
        init_ssm(B);
        B.top = B.xi[ni + 2 * ng - 1] > tree.rr[1];
        B.bottom = B.xi[0] < tree.rr[0];
    }
    // ModCommunication_SetGCAll (single rank)
    for (auto& B : blk) find_gc(B);
    for (auto& B : blk) gc_targets(B);
    gc_sources();
}

void Oracle::init_grid(Block& b) {
    // 3_6/ModBlock.f90:288-438 (iGeometry = 1)
    auto& r = b.rng;
    b.xi.resize(nip); b.xj.resize(njp); b.xk.resize(nkp);
    for (int i = 1 - ng; i <= ni + ng; ++i)
        b.xi[i + ng - 1] = (r[0][0] * (double)((float)(ni - i) + 0.5f) + r[0][1] * (double)((float)i - 0.5f)) / ni;
    for (int j = 1 - ng; j <= nj + ng; ++j)
        b.xj[j + ng - 1] = (r[1][0] * (double)((float)(nj - j) + 0.5f) + r[1][1] * (double)((float)j - 0.5f)) / nj;
    for (int k = 1 - ng; k <= nk + ng; ++k)
        b.xk[k + ng - 1] = (r[2][0] * (double)((float)(nk - k) + 0.5f) + r[2][1] * (double)((float)k - 0.5f)) / nk;
    b.dxi = (r[0][1] - r[0][0]) / ni;
    b.dxj = (r[1][1] - r[1][0]) / nj;
    b.dxk = (r[2][1] - r[2][0]) / nk;
    b.h.resize((size_t)ni * nj * nk);
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                double x = b.xi[i + ng - 1];
                double a = b.dxi, c = x * b.dxj, d = x * std::sin(b.xj[j + ng - 1]) * b.dxk;
                b.h[iidx(i, j, k)] = std::min(std::min(a, c), d);
            }
}

void Oracle::init_ssm(Block& b) {
    // 3_6/ModBlock.f90:188-265
    b.prof.assign((size_t)NPROF * nip, 0.0);
    double o[NPROF];
    for (int i = 0; i < nip; ++i) {
        bg.get_vars(b.xi[i], o);
        for (int p = 0; p < NPROF; ++p) b.prof[(size_t)p * nip + i] = o[p];
    }
    derive_ssm(b);
}

// the block's background arrays from its 1-D profiles (3_6/ModBlock.f90:233-264)
void Oracle::derive_ssm(Block& b) {
    auto P = [&](int p, int i) { return b.prof[(size_t)p * nip + i]; };
    b.gamma1.resize(nip); b.g3m1.resize(nip); b.rho0.resize(nip); b.g_over_rho0.resize(nip);
    b.p0_over_rho0.resize(nip); b.rho0T0.resize(nip); b.heat.resize(nip); b.Xi.resize(nip);
    for (int i = 0; i < nip; ++i) {
        b.gamma1[i] = P(4, i);
        b.g3m1[i] = P(5, i) - 1.0;
        b.rho0[i] = P(1, i);
        b.g_over_rho0[i] = P(0, i) / P(1, i);
        b.p0_over_rho0[i] = P(2, i) / P(1, i);
        b.rho0T0[i] = P(1, i) * P(3, i);
        b.heat[i] = P(6, i) + P(7, i);
        b.Xi[i] = P(8, i);
    }
}

void Oracle::find_gc(Block& b) {
    // 3_6/ModGC.f90:25-51
    b.owner.assign(ncell, -777);
    for (int i = 1 - ng; i <= ni + ng; ++i)
        for (int j = 1 - ng; j <= nj + ng; ++j)
            for (int k = 1 - ng; k <= nk + ng; ++k) {
                double rtp[3] = {b.xi[i + ng - 1], b.xj[j + ng - 1], b.xk[k + ng - 1]};
                if (i < 1 || j < 1 || k < 1 || i > ni || j > nj || k > nk) {
                    const Node* nd = tree.find(rtp, b.yin);
                    if (nd) b.owner[idx(i, j, k)] = nd->leaf_id;
                }
            }
}

void Oracle::gc_targets(Block& b) {
    // 3_6/ModGC.f90:53-147
    std::vector<int> uniq;
    auto ghost = [&](int i, int j, int k) { return i < 1 || i > ni || j < 1 || j > nj || k < 1 || k > nk; };
    for (int i = 1 - ng; i <= ni + ng; ++i)
        for (int j = 1 - ng; j <= nj + ng; ++j)
            for (int k = 1 - ng; k <= nk + ng; ++k)
                if (ghost(i, j, k) && b.owner[idx(i, j, k)] != -777) {
                    int o = b.owner[idx(i, j, k)];
                    if (std::find(uniq.begin(), uniq.end(), o) == uniq.end()) uniq.push_back(o);
                }
    b.targets.resize(uniq.size());
    for (size_t u = 0; u < uniq.size(); ++u) {
        GCList& t = b.targets[u];
        t.other = uniq[u];
        t.other_yin = t.other <= tree.nleaf_yin;
        for (int i = 1 - ng; i <= ni + ng; ++i)
            for (int j = 1 - ng; j <= nj + ng; ++j)
                for (int k = 1 - ng; k <= nk + ng; ++k)
                    if (ghost(i, j, k) && b.owner[idx(i, j, k)] == t.other) {
                        t.ijk.push_back(i); t.ijk.push_back(j); t.ijk.push_back(k);
                        t.x.push_back(b.xi[i + ng - 1]);
                        t.x.push_back(b.xj[j + ng - 1]);
                        t.x.push_back(b.xk[k + ng - 1]);
                    }
    }
}

void Oracle::gc_sources() {
    // 3_6/ModCommunication.f90:111-176 and 258-300 (local path)
    for (auto& B : blk) B.sources.clear();
    for (auto& T : blk)
        for (auto& t : T.targets) {
            Block& S = blk[t.other - 1];
            GCList s;
            s.other = T.id;
            s.other_yin = T.yin;
            s.ijk = t.ijk;
            size_t n = t.ijk.size() / 3;
            s.x.resize(3 * n);
            for (size_t g = 0; g < n; ++g) {
                if (s.other_yin == S.yin) {
                    for (int d = 0; d < 3; ++d) s.x[3 * g + d] = t.x[3 * g + d];
                } else {
                    coord_conv(&t.x[3 * g], &s.x[3 * g]);
                }
            }
            S.sources.push_back(std::move(s));
        }
}

void Oracle::interp(const Block& S, bool rk, const double* x, bool rotate, double* val) const {
    const std::vector<double>& f = rk ? S.urk : S.u;
    double dxi = S.xi[2 + ng - 1] - S.xi[1 + ng - 1];
    double dxj = S.xj[2 + ng - 1] - S.xj[1 + ng - 1];
    double dxk = S.xk[2 + ng - 1] - S.xk[1 + ng - 1];
    // ModMath_1D3D_interpolate_1D1D (3_6/ModMath.f90:250-293)
    double pi_ = (double)((float)(-ng) + 1.0f) + (x[0] - S.xi[0]) / dxi;
    double pj = (double)((float)(-ng) + 1.0f) + (x[1] - S.xj[0]) / dxj;
    double pk = (double)((float)(-ng) + 1.0f) + (x[2] - S.xk[0]) / dxk;
    pi_ = std::max(std::min(pi_, (double)((float)ni + 0.0f)), 1.0);
    pj = std::max(std::min(pj, (double)((float)nj + 0.0f)), 1.0);
    pk = std::max(std::min(pk, (double)((float)nk + 0.0f)), 1.0);
    int i0 = (int)std::floor(pi_), j0 = (int)std::floor(pj), k0 = (int)std::floor(pk);
    double wi = pi_ - i0, wj = pj - j0, wk = pk - k0;
    for (int v = 0; v < nvar; ++v) {
        const double* fv = &f[(size_t)v * ncell];
        val[v] = fv[idx(i0, j0, k0)] * (1. - wi) * (1. - wj) * (1. - wk) +
                 fv[idx(i0 + 1, j0, k0)] * (wi) * (1. - wj) * (1. - wk) +
                 fv[idx(i0, j0 + 1, k0)] * (1. - wi) * (wj) * (1. - wk) +
                 fv[idx(i0, j0, k0 + 1)] * (1. - wi) * (1. - wj) * (wk) +
                 fv[idx(i0 + 1, j0 + 1, k0)] * (wi) * (wj) * (1. - wk) +
                 fv[idx(i0, j0 + 1, k0 + 1)] * (1. - wi) * (wj) * (wk) +
                 fv[idx(i0 + 1, j0, k0 + 1)] * (wi) * (1. - wj) * (wk) +
                 fv[idx(i0 + 1, j0 + 1, k0 + 1)] * (wi) * (wj) * (wk);
    }
    if (rotate) {
        // ModYinYang_VecConv_1D for B then v (3_6/ModCommunication.f90:695-702)
        // B is rotated whenever the layout has B (br_ > 0), as in the reference
        double o[3];
        vec_conv(x, &val[BR], o);
        val[BR] = o[0]; val[BT] = o[1]; val[BP] = o[2];
        vec_conv(x, &val[VR], o);
        val[VR] = o[0]; val[VT] = o[1]; val[VP] = o[2];
    }
}

void Oracle::exchange(bool rk) {
    // 3_6/ModCommunication.f90:678-721 (single rank: every target is local).
    // Source blocks in parallel, as the reference's ranks run them: every
    // ghost cell is written by exactly one entry, and the interpolation reads
    // a source's own ghost cells only with a zero weight. A rank of a sharded
    // run fills the entries whose source and target it owns; the others
    // travel between ranks (orc_interp_entries, orc_write_ghosts).
#pragma omp parallel for schedule(dynamic, 4)
    for (size_t sb = 0; sb < blk.size(); ++sb) {
        if (!owned((int)sb)) continue;
        Block& S = blk[sb];
        for (auto& s : S.sources) {
            if (!owned(s.other - 1)) continue;
            Block& T = blk[s.other - 1];
            std::vector<double>& tgt = rk ? T.urk : T.u;
            size_t n = s.ijk.size() / 3;
            for (size_t g = 0; g < n; ++g) {
                double val[FALCON_NVAR];
                interp(S, rk, &s.x[3 * g], s.other_yin != S.yin, val);
                int ti = s.ijk[3 * g], tj = s.ijk[3 * g + 1], tk = s.ijk[3 * g + 2];
                for (int v = 0; v < nvar; ++v) tgt[(size_t)v * ncell + idx(ti, tj, tk)] = val[v];
            }
        }
    }
}

void Oracle::boundary(Block& b, std::vector<double>& p) {
    // 3_6/ModBoundary.f90:10-55: whole (j,k) planes including their ghosts
    auto plane = [&](int v, int i_dst, int i_src, double sgn) {
        for (int k = 1 - ng; k <= nk + ng; ++k)
            for (int j = 1 - ng; j <= nj + ng; ++j) {
                double s = p[(size_t)v * ncell + idx(i_src, j, k)];
                p[(size_t)v * ncell + idx(i_dst, j, k)] = sgn > 0 ? s : -s;
            }
    };
    bool B = cfg.phys.if_involve_B != 0;
    if (b.top) {
        for (int i = ni + 1; i <= ni + ng; ++i) {
            plane(RHO1, i, 2 * ni + 1 - i, 1); plane(VT, i, 2 * ni + 1 - i, 1);
            plane(VP, i, 2 * ni + 1 - i, 1); plane(S1, i, 2 * ni + 1 - i, 1);
            plane(VR, i, 2 * ni + 1 - i, -1);
        }
        if (B)
            for (int i = ni + 1; i <= ni + ng; ++i) {
                plane(BR, i, 2 * ni + 1 - i, 1); plane(BT, i, 2 * ni + 1 - i, -1);
                plane(BP, i, 2 * ni + 1 - i, -1);
            }
    }
    if (b.bottom) {
        for (int i = -ng + 1; i <= 0; ++i) {
            plane(RHO1, i, 1 - i, 1); plane(VT, i, 1 - i, 1);
            plane(VP, i, 1 - i, 1); plane(S1, i, 1 - i, 1);
            plane(VR, i, 1 - i, -1);
        }
        if (B)
            for (int i = -ng + 1; i <= 0; ++i) {
                plane(BR, i, 1 - i, -1); plane(BT, i, 1 - i, 1); plane(BP, i, 1 - i, 1);
            }
    }
}

// ---- ModDerivative / ModSpherical ------------------------------------------
typedef std::vector<double> Arr;

struct Ops {
    const Oracle& o;
    const Block& b;
    double c12[3];
    Ops(const Oracle& o_, const Block& b_) : o(o_), b(b_) {
        const double c = (double)(1.0f / 12.0f);   // 1./12. is a default-real constant
        c12[0] = c / b.dxi; c12[1] = c / b.dxj; c12[2] = c / b.dxk;
    }
    int ni() const { return o.ni; }
    // ModDerivative_1st_O4_3D (3_6/ModDerivative.f90:5-34): padded -> interior
    Arr D(const Arr& f, int dir) const {
        Arr out((size_t)o.ni * o.nj * o.nk);
        int si = 1, sj = o.nip, sk = o.nip * o.njp;
        int s = dir == 1 ? si : dir == 2 ? sj : sk;
        double c = c12[dir - 1];
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    int m = o.idx(i, j, k);
                    out[o.iidx(i, j, k)] = c * (((-f[m + 2 * s] + 8. * f[m + s]) - 8. * f[m - s]) + f[m - 2 * s]);
                }
        return out;
    }
    Arr comp(const Arr& p, int v) const {
        return Arr(p.begin() + (size_t)v * o.ncell, p.begin() + (size_t)(v + 1) * o.ncell);
    }
    double rr(int i) const { return b.xi[i + o.ng - 1]; }
    double tt(int j) const { return b.xj[j + o.ng - 1]; }
    // ModSpherical_A_dot_Grad_f (3_6/ModSpherical.f90:241-279)
    Arr a_dot_grad(const Arr& A1, const Arr& A2, const Arr& A3, const Arr& f) const {
        Arr d1 = D(f, 1), d2 = D(f, 2), d3 = D(f, 3), out(d1.size());
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    int m = o.idx(i, j, k), q = o.iidx(i, j, k);
                    double rinv = 1. / rr(i), sinv = 1. / std::sin(tt(j));
                    double adg = A1[m] * d1[q];
                    double tmp = A2[m] * d2[q];
                    adg = adg + tmp * rinv;
                    tmp = A3[m] * d3[q];
                    tmp = tmp * rinv;
                    adg = adg + sinv * tmp;
                    out[q] = adg;
                }
        return out;
    }
    // ModSpherical_curl (3_6/ModSpherical.f90:38-102)
    void curl(const Arr& A1, const Arr& A2, const Arr& A3, Arr& c1, Arr& c2, Arr& c3) const {
        Arr At_r(o.ncell), Ap_r(o.ncell), Ar_s(o.ncell), Ap_s(o.ncell);
        for (int k = 1 - o.ng; k <= o.nk + o.ng; ++k)
            for (int j = 1 - o.ng; j <= o.nj + o.ng; ++j)
                for (int i = 1 - o.ng; i <= o.ni + o.ng; ++i) {
                    int m = o.idx(i, j, k);
                    double st = std::sin(tt(j));
                    At_r[m] = A2[m] * rr(i);
                    Ap_r[m] = A3[m] * rr(i);
                    Ar_s[m] = A1[m] / st;
                    Ap_s[m] = A3[m] * st;
                }
        Arr a = D(Ap_s, 2), bb = D(A2, 3);
        c1.resize(a.size()); c2.resize(a.size()); c3.resize(a.size());
        for (size_t q = 0; q < a.size(); ++q) c1[q] = a[q] - bb[q];
        a = D(Ar_s, 3); bb = D(Ap_r, 1);
        for (size_t q = 0; q < a.size(); ++q) c2[q] = a[q] - bb[q];
        a = D(At_r, 1); bb = D(A1, 2);
        for (size_t q = 0; q < a.size(); ++q) c3[q] = a[q] - bb[q];
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    int q = o.iidx(i, j, k);
                    double rinv = 1. / rr(i);
                    c1[q] = c1[q] * rinv; c2[q] = c2[q] * rinv; c3[q] = c3[q] * rinv;
                }
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    int q = o.iidx(i, j, k);
                    c1[q] = c1[q] * (1. / std::sin(tt(j)));
                }
    }
    // ModSpherical_div (3_6/ModSpherical.f90:104-159)
    Arr div(const Arr& A1, const Arr& A2, const Arr& A3) const {
        Arr S1(o.ncell), S2(o.ncell);
        for (int k = 1 - o.ng; k <= o.nk + o.ng; ++k)
            for (int j = 1 - o.ng; j <= o.nj + o.ng; ++j)
                for (int i = 1 - o.ng; i <= o.ni + o.ng; ++i) {
                    int m = o.idx(i, j, k);
                    double r = rr(i);
                    S1[m] = A1[m] * (r * r);
                    S2[m] = A2[m] * std::sin(tt(j));
                }
        Arr d = D(S1, 1);
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    double r = rr(i);
                    d[o.iidx(i, j, k)] = d[o.iidx(i, j, k)] * (1. / (r * r));
                }
        Arr d23 = D(S2, 2), d3 = D(A3, 3);
        for (size_t q = 0; q < d23.size(); ++q) d23[q] = d23[q] + d3[q];
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    int q = o.iidx(i, j, k);
                    d23[q] = d23[q] * (1. / std::sin(tt(j)));
                }
        for (int k = 1; k <= o.nk; ++k)
            for (int j = 1; j <= o.nj; ++j)
                for (int i = 1; i <= o.ni; ++i) {
                    int q = o.iidx(i, j, k);
                    d23[q] = d23[q] * (1. / rr(i));
                }
        for (size_t q = 0; q < d.size(); ++q) d[q] = d[q] + d23[q];
        return d;
    }
};

void Oracle::equation(Block& b, const std::vector<double>& p) {
    // ModEquation_Dynamo (3_6/ModEquation.f90:24-162)
    Ops op(*this, b);
    const int nint = ni * nj * nk;
    Arr rho1 = op.comp(p, RHO1), vr = op.comp(p, VR), vt = op.comp(p, VT), vp = op.comp(p, VP);
    Arr br = op.comp(p, BR), bt = op.comp(p, BT), bp = op.comp(p, BP), s1 = op.comp(p, S1);
    auto I = [&](int i, int j, int k) { return idx(i, j, k); };
    // Get_p1 (:40-46), over the padded block
    b.p1.assign(ncell, 0.0);
    for (int k = 1 - ng; k <= nk + ng; ++k)
        for (int j = 1 - ng; j <= nj + ng; ++j)
            for (int i = 1 - ng; i <= ni + ng; ++i) {
                int m = I(i, j, k), r = i + ng - 1;
                b.p1[m] = b.gamma1[r] * b.p0_over_rho0[r] * rho1[m] + b.g3m1[r] * b.rho0T0[r] * s1[m];
            }
    Arr& R = b.R;
    auto Rv = [&](int v, int q) -> double& { return R[(size_t)v * nint + q]; };
    // Mass_Conservation (:50-61)
    {
        Arr t1(ncell), t2(ncell), t3(ncell);
        for (int k = 1 - ng; k <= nk + ng; ++k)
            for (int j = 1 - ng; j <= nj + ng; ++j)
                for (int i = 1 - ng; i <= ni + ng; ++i) {
                    int m = I(i, j, k), r = i + ng - 1;
                    t1[m] = b.rho0[r] * vr[m]; t2[m] = b.rho0[r] * vt[m]; t3[m] = b.rho0[r] * vp[m];
                }
        Arr d = op.div(t1, t2, t3);
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    int q = iidx(i, j, k), r = i + ng - 1;
                    double x = b.Xi[r];
                    Rv(RHO1, q) = -(1.0 / (x * x) * d[q]);
                }
    }
    // Inertial_Force (:66-74): -A_dot_nabla_B(v, v) (3_6/ModSpherical.f90:281-343)
    {
        Arr a1 = op.a_dot_grad(vr, vt, vp, vr);
        Arr a2 = op.a_dot_grad(vr, vt, vp, vt);
        Arr a3 = op.a_dot_grad(vr, vt, vp, vp);
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    int q = iidx(i, j, k), m = I(i, j, k);
                    double rinv = 1. / op.rr(i);
                    double t = op.tt(j);
                    double cot = std::cos(t) / std::sin(t);
                    double tmp = -(vt[m] * vt[m]) - vp[m] * vp[m];
                    a1[q] = a1[q] + tmp * rinv;
                    tmp = -(vp[m] * vp[m]);
                    tmp = tmp * cot;
                    tmp = tmp + vt[m] * vr[m];
                    a2[q] = a2[q] + tmp * rinv;
                    tmp = vp[m] * vt[m];
                    tmp = tmp * cot;
                    tmp = tmp + vp[m] * vr[m];
                    a3[q] = a3[q] + tmp * rinv;
                    Rv(VR, q) = -a1[q]; Rv(VT, q) = -a2[q]; Rv(VP, q) = -a3[q];
                }
    }
    // Pressure_Gradient (:79-92): Grad_f (3_6/ModSpherical.f90:201-239)
    {
        Arr g1 = op.D(b.p1, 1), g2 = op.D(b.p1, 2), g3 = op.D(b.p1, 3);
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    int q = iidx(i, j, k), r = i + ng - 1;
                    double rinv = 1. / op.rr(i), sinv = 1. / std::sin(op.tt(j));
                    double G2 = g2[q] * rinv;
                    double G3 = g3[q] * rinv;
                    G3 = G3 * sinv;
                    Rv(VR, q) = Rv(VR, q) - g1[q] / b.rho0[r];
                    Rv(VT, q) = Rv(VT, q) - G2 / b.rho0[r];
                    Rv(VP, q) = Rv(VP, q) - G3 / b.rho0[r];
                }
    }
    bool withB = cfg.phys.if_involve_B != 0;
    // Lorentz_Force (:97-116)
    if (withB) {
        Arr c1, c2, c3;
        op.curl(br, bt, bp, c1, c2, c3);
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    int q = iidx(i, j, k), m = I(i, j, k), r = i + ng - 1;
                    double x1 = c2[q] * bp[m] - c3[q] * bt[m];
                    double x2 = c3[q] * br[m] - c1[q] * bp[m];
                    double x3 = c1[q] * bt[m] - c2[q] * br[m];
                    Rv(VR, q) = Rv(VR, q) + x1 / b.rho0[r];
                    Rv(VT, q) = Rv(VT, q) + x2 / b.rho0[r];
                    Rv(VP, q) = Rv(VP, q) + x3 / b.rho0[r];
                }
    }
    // Gravity (:121-127)
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                int q = iidx(i, j, k), r = i + ng - 1;
                Rv(VR, q) = Rv(VR, q) - b.g_over_rho0[r] * rho1[I(i, j, k)];
            }
    // Entropy_Advection (:132-140) and Entropy_Heating (:145-151)
    {
        Arr a = op.a_dot_grad(vr, vt, vp, s1);
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    int q = iidx(i, j, k), r = i + ng - 1;
                    Rv(S1, q) = -a[q];
                    Rv(S1, q) = Rv(S1, q) + cfg.phys.heating_ratio * b.heat[r] / b.rho0T0[r];
                }
    }
    // Induction_Equation (:154-162)
    if (withB) {
        Arr e1(ncell), e2(ncell), e3(ncell);
        for (int m = 0; m < ncell; ++m) {
            e1[m] = vt[m] * bp[m] - vp[m] * bt[m];
            e2[m] = vp[m] * br[m] - vr[m] * bp[m];
            e3[m] = vr[m] * bt[m] - vt[m] * br[m];
        }
        Arr c1, c2, c3;
        op.curl(e1, e2, e3, c1, c2, c3);
        for (int q = 0; q < nint; ++q) { Rv(BR, q) = c1[q]; Rv(BT, q) = c2[q]; Rv(BP, q) = c3[q]; }
    }
    for (int q = 0; q < nint; ++q) Rv(PSI, q) = 0.0;
    if (withB && cfg.phys.divb_option == 1) glm(b, p);
    if (withB && cfg.phys.divb_option == 2) powell(b, p);
}

void Oracle::glm(Block& b, const std::vector<double>& p) {
    // ModDivB_GLM (3_6/ModDivB.f90:13-38): dB/dt += -grad(psi);
    // dpsi/dt = -v_wave^2 div(B) - v_wave/h_LLL psi, v_wave from the step start
    Ops op(*this, b);
    const int nint = ni * nj * nk;
    auto Rv = [&](int v, int q) -> double& { return b.R[(size_t)v * nint + q]; };
    Arr br = op.comp(p, BR), bt = op.comp(p, BT), bp = op.comp(p, BP), psi = op.comp(p, PSI);
    Arr dvb = op.div(br, bt, bp);
    // ModSpherical_Grad_f (3_6/ModSpherical.f90:201-239)
    Arr g1 = op.D(psi, 1), g2 = op.D(psi, 2), g3 = op.D(psi, 3);
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const int q = iidx(i, j, k);
                const double rinv = 1. / op.rr(i), sinv = 1. / std::sin(op.tt(j));
                double G2 = g2[q] * rinv;
                double G3 = g3[q] * rinv;
                G3 = G3 * sinv;
                Rv(BR, q) = Rv(BR, q) - g1[q];
                Rv(BT, q) = Rv(BT, q) - G2;
                Rv(BP, q) = Rv(BP, q) - G3;
                const double w = b.vwave[q];
                Rv(PSI, q) = -(w * w * dvb[q]) - w / b.h[q] * psi[idx(i, j, k)];
            }
}

void Oracle::powell(Block& b, const std::vector<double>& p) {
    // Powell source term of 3_5/ModEquation.f90:169-176: dB_i/dt += -(div B) v_i,
    // with 3_6's ModSpherical_div; applied after the induction term
    Ops op(*this, b);
    const int nint = ni * nj * nk;
    Arr dvb = op.div(op.comp(p, BR), op.comp(p, BT), op.comp(p, BP));
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const int q = iidx(i, j, k), m = idx(i, j, k);
                for (int c = 0; c < 3; ++c)
                    b.R[(size_t)(BR + c) * nint + q] =
                        b.R[(size_t)(BR + c) * nint + q] - dvb[q] * p[(size_t)(VR + c) * ncell + m];
            }
}

// ModLinReconstruct_minmod one value (3_6/ModLinReconstruct.f90:5-49)
static inline double minmod(double ul, double u, double ur) {
    double a = (ur - ul) * 0.5;
    double b = 2.0 * (ur - u);
    double c = 2.0 * (u - ul);
    double s = std::copysign(0.5, std::fmax(0.0, a * b) * std::fmax(0.0, b * c) * 1.e10 - (double)1.e-30f);
    double m = std::fmin(std::fmin(std::fabs(a), std::fabs(b)), std::fabs(c));
    return (s + 0.5) * std::copysign(m, a);
}

void Oracle::diffusion(Block& b, const std::vector<double>& p) {
    // ModDiffusion_Aritificial_1 with h=2 (3_6/ModDiffusion.f90:9-150)
    const int nint = ni * nj * nk;
    Arr cs(ncell);
    for (int k = 1 - ng; k <= nk + ng; ++k)
        for (int j = 1 - ng; j <= nj + ng; ++j)
            for (int i = 1 - ng; i <= ni + ng; ++i) {
                int r = i + ng - 1;
                cs[idx(i, j, k)] = 1. / b.Xi[r] * std::sqrt(b.gamma1[r] * b.p0_over_rho0[r]);
            }
    const double h = 2.0;
    for (int dir = 1; dir <= 3; ++dir) {
        int s = dir == 1 ? 1 : dir == 2 ? nip : nip * njp;
        const double* vdir = &p[(size_t)(dir) * ncell];   // vr, vt, vp are variables 2,3,4
        for (int v = 0; v < nvar; ++v) {
            const double* f = &p[(size_t)v * ncell];
            for (int k = 1; k <= nk; ++k)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        int m = idx(i, j, k);
                        double fl[2];
                        for (int side = 0; side < 2; ++side) {
                            // face between cells mR = m + side*s and mL = mR - s
                            int mR = m + side * s, mL = mR - s;
                            double dR = minmod(f[mR - s], f[mR], f[mR + s]);
                            double dL = minmod(f[mL - s], f[mL], f[mL + s]);
                            double num = ((f[mR] - dR * 0.5) - f[mL]) - dL * 0.5;
                            double phi = std::fmax(0.0, 1.0 + h * (num / (f[mR] - f[mL]) - 1.0));
                            double flux = -(0.5 * phi * num);
                            double cR = std::fabs(vdir[mR]) + cs[mR], cL = std::fabs(vdir[mL]) + cs[mL];
                            flux = flux * (cR + cL) * 0.5;
                            fl[side] = flux;
                        }
                        int q = iidx(i, j, k);
                        double den;
                        if (dir == 1) den = b.dxi;
                        else if (dir == 2) den = b.dxj * b.xi[i + ng - 1];
                        else den = b.dxk * b.xi[i + ng - 1] * std::sin(b.xj[j + ng - 1]);
                        b.R[(size_t)v * nint + q] = b.R[(size_t)v * nint + q] + (fl[0] - fl[1]) / den;
                    }
        }
    }
}

void Oracle::wave_speed(Block& b) {
    // 3_6/ModWaveSpeed.f90:8-27 (reads primitive_IV)
    b.vwave.assign((size_t)ni * nj * nk, 0.0);
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                int m = idx(i, j, k), r = i + ng - 1;
                const double* u = b.u.data();
                double vr = u[VR * ncell + m], vt = u[VT * ncell + m], vp = u[VP * ncell + m];
                double w = 1. / b.Xi[r] * std::sqrt(b.gamma1[r] * b.p0_over_rho0[r]) +
                           std::sqrt(vr * vr + vt * vt + vp * vp);
                if (cfg.phys.if_involve_B) {
                    double x = u[BR * ncell + m], y = u[BT * ncell + m], z = u[BP * ncell + m];
                    w = w + std::sqrt(x * x + y * y + z * z) / std::sqrt(b.rho0[r]);
                }
                b.vwave[iidx(i, j, k)] = w;
            }
}

double Oracle::timestep() {
    // 3_6/ModTimeStep.f90:10-30
    double d = (double)1.e20f;
    for (size_t ib = 0; ib < blk.size(); ++ib) {
        if (!owned((int)ib)) continue;
        const Block& b = blk[ib];
        double m = INFINITY;
        for (int q = 0; q < ni * nj * nk; ++q) m = std::min(m, b.h[q] / b.vwave[q]);
        double d1 = cfg.phys.cfl * m;
        d = std::min(d, d1);
    }
    return d;
}

void Oracle::step() {
    // ModAdvance_rk4 (3_6/ModAdvance.f90:18-112)
    const int nint = ni * nj * nk;
    const int nb = (int)blk.size();
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < nb; ++b) wave_speed(blk[b]);
    dt = timestep();
    for (int rk = 1; rk <= 4; ++rk) {
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nb; ++ib) {
            Block& b = blk[ib];
            std::vector<double>& p = rk > 1 ? b.urk : b.u;
            boundary(b, p);
            equation(b, p);
            std::vector<double>& out = rk < 4 ? b.urk : b.u;
            const double div = (double)(5.0f - (float)rk);
            for (int v = 0; v < nvar; ++v)
                for (int k = 1; k <= nk; ++k)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            int m = (int)((size_t)v * ncell) + idx(i, j, k);
                            out[m] = b.u[m] + dt * b.R[(size_t)v * nint + iidx(i, j, k)] / div;
                        }
        }
        exchange(rk < 4);
    }
#pragma omp parallel for schedule(dynamic)
    for (int ib = 0; ib < nb; ++ib) {
        Block& b = blk[ib];
        std::fill(b.R.begin(), b.R.end(), 0.0);
        diffusion(b, b.u);
        for (int v = 0; v < nvar; ++v)
            for (int k = 1; k <= nk; ++k)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        int m = (int)((size_t)v * ncell) + idx(i, j, k);
                        b.u[m] = b.u[m] + 0.5 * dt * b.R[(size_t)v * nint + iidx(i, j, k)];
                    }
    }
    exchange(false);
}

// One phase of step(): 0 wave speed + dt, 1..4 RK stage, 5 diffusion.
void Oracle::phase(int ph) {
    const int nint = ni * nj * nk;
    const int nb = (int)blk.size();
    if (ph == 0) {
#pragma omp parallel for schedule(dynamic)
        for (int b = 0; b < nb; ++b)
            if (owned(b)) wave_speed(blk[b]);
        dt = timestep();
        return;
    }
    if (ph <= 4) {
        const int rk = ph;
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nb; ++ib) {
            if (!owned(ib)) continue;
            Block& b = blk[ib];
            std::vector<double>& p = rk > 1 ? b.urk : b.u;
            boundary(b, p);
            equation(b, p);
            std::vector<double>& out = rk < 4 ? b.urk : b.u;
            const double div = (double)(5.0f - (float)rk);
            for (int v = 0; v < nvar; ++v)
                for (int k = 1; k <= nk; ++k)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            int m = (int)((size_t)v * ncell) + idx(i, j, k);
                            out[m] = b.u[m] + dt * b.R[(size_t)v * nint + iidx(i, j, k)] / div;
                        }
        }
        exchange(rk < 4);
        return;
    }
#pragma omp parallel for schedule(dynamic)
    for (int ib = 0; ib < nb; ++ib) {
        if (!owned(ib)) continue;
        Block& b = blk[ib];
        std::fill(b.R.begin(), b.R.end(), 0.0);
        diffusion(b, b.u);
        for (int v = 0; v < nvar; ++v)
            for (int k = 1; k <= nk; ++k)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        int m = (int)((size_t)v * ncell) + idx(i, j, k);
                        b.u[m] = b.u[m] + 0.5 * dt * b.R[(size_t)v * nint + iidx(i, j, k)];
                    }
    }
    exchange(false);
}

}  // namespace orc

// ---- ModSave_AllCells (3_6/ModSavePlot.f90:520-650) ------------------------
namespace orc {
// Fortran ES16.8 (gfortran): d.ddddddddE+dd right-justified in 16 columns,
// the E dropped before a three-digit exponent
static std::string fortran_es16_8(double x) {
    char b[64];
    if (std::isnan(x)) std::snprintf(b, sizeof b, "NaN");
    else if (std::isinf(x)) std::snprintf(b, sizeof b, "%s", x > 0 ? "Infinity" : "-Infinity");
    else std::snprintf(b, sizeof b, "%.8E", x);
    std::string t(b);
    const size_t e = t.find('E');
    if (e != std::string::npos && t.size() - e - 2 == 3) t.erase(e, 1);
    if (t.size() > 16) return std::string(16, '*');
    return std::string(16 - t.size(), ' ') + t;
}
static std::string fortran_i8_zero(long v) {
    char b[32];
    std::snprintf(b, sizeof b, "%8ld", v);
    std::string t(b);
    for (char& c : t)
        if (c == ' ') c = '0';
    return t;
}
}  // namespace orc

static int orc_save_allcells_impl(orc::Oracle& o, const char* directory, int step) {
    using namespace orc;
    const std::string dir = std::string(directory) + "/AllCells_" + fortran_i8_zero(step);
    std::filesystem::create_directories(dir);
    FILE* f = std::fopen((dir + "/info.dat").c_str(), "w");
    if (!f) return -1;
    std::fprintf(f, "nBlocks = %d\n", (int)o.blk.size());
    std::fprintf(f, "ni = %d\nnj = %d\nnk = %d\n", o.ni, o.nj, o.nk);
    std::fprintf(f, "nVarsTotal = %d\n", o.nvar + 3);
    std::fprintf(f, "VARIABLES = \"X [Rs]\", \"Y [Rs]\", \"Z [Rs]\", \"Rho1\", \"Vx\", \"Vy\", \"Vz\", \"Bx\", "
                    "\"By\", \"Bz\", \"S1\", \"PHI\"\n");
    std::fclose(f);
    const double rsun = (double)6.955e10f;   // R_sun__CGS (3_6/ModConst.f90:5)
    const int ni = o.ni, nj = o.nj, nk = o.nk, nv = o.nvar;
    for (const Block& B : o.blk) {
        // corner values (3_6/ModSavePlot.f90:572-582)
        std::vector<double> cor((size_t)(ni + 1) * (nj + 1) * (nk + 1) * nv);
        auto p = [&](int v, int i, int j, int k) { return B.u[(size_t)v * o.ncell + o.idx(i, j, k)]; };
        size_t q = 0;
        for (int k = 1; k <= nk + 1; ++k)
            for (int j = 1; j <= nj + 1; ++j)
                for (int i = 1; i <= ni + 1; ++i, ++q)
                    for (int v = 0; v < nv; ++v)
                        cor[q * nv + v] = 0.125 * (p(v, i - 1, j - 1, k - 1) + p(v, i, j - 1, k - 1) +
                                                   p(v, i - 1, j, k - 1) + p(v, i, j, k - 1) +
                                                   p(v, i - 1, j - 1, k) + p(v, i, j - 1, k) +
                                                   p(v, i - 1, j, k) + p(v, i, j, k));
        // face coordinates (3_6/ModBlock.f90:320-322)
        std::vector<double> xf(ni + 1), yf(nj + 1), zf(nk + 1);
        for (int i = 1; i <= ni + 1; ++i) xf[i - 1] = (B.rng[0][0] * (ni + 1 - i) + B.rng[0][1] * (i - 1)) / ni;
        for (int j = 1; j <= nj + 1; ++j) yf[j - 1] = (B.rng[1][0] * (nj + 1 - j) + B.rng[1][1] * (j - 1)) / nj;
        for (int k = 1; k <= nk + 1; ++k) zf[k - 1] = (B.rng[2][0] * (nk + 1 - k) + B.rng[2][1] * (k - 1)) / nk;
        f = std::fopen((dir + "/Block_" + fortran_i8_zero(B.id) + ".dat").c_str(), "w");
        if (!f) return -1;
        q = 0;
        for (int k = 1; k <= nk + 1; ++k)
            for (int j = 1; j <= nj + 1; ++j)
                for (int i = 1; i <= ni + 1; ++i, ++q) {
                    const double r = xf[i - 1], th = yf[j - 1], ph = zf[k - 1];
                    const double sth = std::sin(th), cth = std::cos(th), sph = std::sin(ph), cph = std::cos(ph);
                    double xyz[3];
                    if (B.yin) {
                        xyz[0] = r * sth * cph;
                        xyz[1] = r * sth * sph;
                        xyz[2] = r * cth;
                    } else {
                        xyz[0] = -(r * sth * cph);
                        xyz[1] = r * cth;
                        xyz[2] = r * sth * sph;
                    }
                    for (double& c : xyz) c = c / rsun;
                    double vo[FALCON_NVAR];
                    for (int v = 0; v < nv; ++v) vo[v] = cor[q * nv + v];
                    for (int a : {VR, BR}) {
                        const double vx = vo[a] * sth * cph + vo[a + 1] * cth * cph - vo[a + 2] * sph;
                        const double vy = vo[a] * sth * sph + vo[a + 1] * cth * sph + vo[a + 2] * cph;
                        const double vz = vo[a] * cth - vo[a + 1] * sth;
                        if (B.yin) { vo[a] = vx; vo[a + 1] = vy; vo[a + 2] = vz; }
                        else { vo[a] = -vx; vo[a + 1] = vz; vo[a + 2] = vy; }
                    }
                    std::string line;
                    for (double c : xyz) line += fortran_es16_8(c);
                    for (int v = 0; v < nv; ++v) line += fortran_es16_8(vo[v]);
                    line += '\n';
                    std::fputs(line.c_str(), f);
                }
        std::fclose(f);
    }
    return 0;
}

// ---- C API used by the tests and by bench.py's CPU baseline -------------
using orc::Oracle;

extern "C" {

void* orc_create(const falcon_config* cfg) {
    Oracle* o = new Oracle();
    o->cfg = *cfg;
    o->build();
    return o;
}
void orc_destroy(void* h) { delete (Oracle*)h; }
int orc_num_blocks(void* h, int32_t* nb, int32_t* nyin) {
    Oracle* o = (Oracle*)h;
    *nb = (int32_t)o->blk.size();
    *nyin = o->tree.nleaf_yin;
    return 0;
}
int orc_block_ranges(void* h, double* out) {
    Oracle* o = (Oracle*)h;
    for (size_t b = 0; b < o->blk.size(); ++b) std::memcpy(out + 6 * b, o->blk[b].rng, 6 * sizeof(double));
    return 0;
}
int orc_block_flags(void* h, int32_t* out) {
    Oracle* o = (Oracle*)h;
    for (size_t b = 0; b < o->blk.size(); ++b)
        out[b] = (o->blk[b].yin ? 1 : 0) | (o->blk[b].top ? 2 : 0) | (o->blk[b].bottom ? 4 : 0);
    return 0;
}
int orc_block_grid(void* h, int32_t b, double* xi, double* xj, double* xk, double* d) {
    Oracle* o = (Oracle*)h;
    const auto& B = o->blk[b];
    std::memcpy(xi, B.xi.data(), B.xi.size() * sizeof(double));
    std::memcpy(xj, B.xj.data(), B.xj.size() * sizeof(double));
    std::memcpy(xk, B.xk.data(), B.xk.size() * sizeof(double));
    d[0] = B.dxi; d[1] = B.dxj; d[2] = B.dxk;
    return 0;
}
int orc_get_background(void* h, double* out) {
    Oracle* o = (Oracle*)h;
    size_t n = (size_t)FALCON_NPROF * o->nip;
    for (size_t b = 0; b < o->blk.size(); ++b) std::memcpy(out + n * b, o->blk[b].prof.data(), n * sizeof(double));
    return 0;
}
// the driver's own profiles [b][NPROF][nip] in place of the polytrope's
int orc_set_background(void* h, const double* in) {
    Oracle* o = (Oracle*)h;
    size_t n = (size_t)FALCON_NPROF * o->nip;
    for (size_t b = 0; b < o->blk.size(); ++b) {
        std::memcpy(o->blk[b].prof.data(), in + n * b, n * sizeof(double));
        o->derive_ssm(o->blk[b]);
    }
    return 0;
}
int64_t orc_ghost_count(void* h) {
    Oracle* o = (Oracle*)h;
    int64_t n = 0;
    for (auto& b : o->blk)
        for (auto& t : b.targets) n += (int64_t)(t.ijk.size() / 3);
    return n;
}
// uncovered non-radial ghosts (owner -777 although the cell centre lies inside the radial range)
int64_t orc_uncovered_ghosts(void* h) {
    Oracle* o = (Oracle*)h;
    int64_t n = 0;
    for (auto& b : o->blk)
        for (int i = 1 - o->ng; i <= o->ni + o->ng; ++i)
            for (int j = 1 - o->ng; j <= o->nj + o->ng; ++j)
                for (int k = 1 - o->ng; k <= o->nk + o->ng; ++k) {
                    bool ghost = i < 1 || i > o->ni || j < 1 || j > o->nj || k < 1 || k > o->nk;
                    double r = b.xi[i + o->ng - 1];
                    if (ghost && b.owner[o->idx(i, j, k)] == -777 && r > o->tree.rr[0] && r < o->tree.rr[1]) ++n;
                }
    return n;
}
// Export the map in the reference order: target block, its GC_targets, i-j-k order.
int orc_ghost_map(void* h, falcon_ghost_entry* out, int64_t cap) {
    Oracle* o = (Oracle*)h;
    int64_t n = 0;
    for (auto& T : o->blk)
        for (auto& t : T.targets) {
            const orc::Block& S = o->blk[t.other - 1];
            // the source-frame coordinates live in the source's GC_sources list
            const orc::GCList* s = nullptr;
            for (auto& c : S.sources) if (c.other == T.id) { s = &c; break; }
            size_t m = t.ijk.size() / 3;
            for (size_t g = 0; g < m; ++g) {
                if (n >= cap) return -1;
                falcon_ghost_entry& e = out[n++];
                e.tblock = T.id - 1;
                e.ti = t.ijk[3 * g]; e.tj = t.ijk[3 * g + 1]; e.tk = t.ijk[3 * g + 2];
                e.sblock = t.other - 1; e.pad_ = 0;
                for (int d = 0; d < 3; ++d) e.src_x[d] = s->x[3 * g + d];
            }
        }
    return 0;
}
int orc_set_state(void* h, const double* u) {
    Oracle* o = (Oracle*)h;
    size_t n = (size_t)o->nvar * o->ncell;
    for (size_t b = 0; b < o->blk.size(); ++b) {
        std::memcpy(o->blk[b].u.data(), u + n * b, n * sizeof(double));
        o->blk[b].urk = o->blk[b].u;   // ModInitiation copies primitive_IV to primitive_rk_IV
    }
    return 0;
}
int orc_get_state(void* h, double* u) {
    Oracle* o = (Oracle*)h;
    size_t n = (size_t)o->nvar * o->ncell;
    for (size_t b = 0; b < o->blk.size(); ++b) std::memcpy(u + n * b, o->blk[b].u.data(), n * sizeof(double));
    return 0;
}
int orc_phase(void* h, int32_t ph) { ((Oracle*)h)->phase(ph); return 0; }
double orc_dt(void* h) { return ((Oracle*)h)->dt; }
// ---- block sharding (a rank of a multi-rank run) -----------------------------
int orc_set_owned(void* h, int32_t first, int32_t last) {
    Oracle* o = (Oracle*)h;
    o->own_first = first;
    o->own_last = last;
    return 0;
}
// the step's dt after the MIN over ranks (3_6/ModAdvance.f90:48)
int orc_set_dt(void* h, double dt) { ((Oracle*)h)->dt = dt; return 0; }
// values of ghost entries ent[n][5] = (target block, ti, tj, tk, source block)
// (0-based blocks, Fortran cell indices) with source-frame centres x[n][3],
// from the sources' stage buffer (rk) or state: out[n][nvar]
int orc_interp_entries(void* h, int32_t rk, const int32_t* ent, const double* x, int64_t n, double* out) {
    Oracle* o = (Oracle*)h;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; ++e) {
        const orc::Block& S = o->blk[ent[5 * e + 4]];
        const orc::Block& T = o->blk[ent[5 * e]];
        o->interp(S, rk != 0, x + 3 * e, T.yin != S.yin, out + (size_t)o->nvar * e);
    }
    return 0;
}
// write ghost values vals[n][nvar] into the target cells of ent[n][5]
int orc_write_ghosts(void* h, int32_t rk, const int32_t* ent, int64_t n, const double* vals) {
    Oracle* o = (Oracle*)h;
    for (int64_t e = 0; e < n; ++e) {
        orc::Block& T = o->blk[ent[5 * e]];
        std::vector<double>& tgt = rk ? T.urk : T.u;
        const int c = o->idx(ent[5 * e + 1], ent[5 * e + 2], ent[5 * e + 3]);
        for (int v = 0; v < o->nvar; ++v) tgt[(size_t)v * o->ncell + c] = vals[(size_t)o->nvar * e + v];
    }
    return 0;
}
int orc_get_stage_state(void* h, double* u) {
    Oracle* o = (Oracle*)h;
    size_t n = (size_t)o->nvar * o->ncell;
    for (size_t b = 0; b < o->blk.size(); ++b) std::memcpy(u + n * b, o->blk[b].urk.data(), n * sizeof(double));
    return 0;
}
int orc_save_allcells(void* h, const char* directory, int32_t step) {
    return orc_save_allcells_impl(*(Oracle*)h, directory, step);
}
int orc_exchange(void* h) { ((Oracle*)h)->exchange(false); return 0; }
int orc_timestep(void* h, double* dt) {
    Oracle* o = (Oracle*)h;
    for (auto& b : o->blk) o->wave_speed(b);
    *dt = o->timestep();
    return 0;
}
int orc_step(void* h, double* dt) {
    Oracle* o = (Oracle*)h;
    o->step();
    if (dt) *dt = o->dt;
    return 0;
}
// single-block RHS on an arbitrary padded state (used by known-answer tests)
int orc_block_rhs(void* h, int32_t b, const double* p, double* R) {
    Oracle* o = (Oracle*)h;
    orc::Block& B = o->blk[b];
    std::vector<double> pp(p, p + (size_t)o->nvar * o->ncell);
    o->equation(B, pp);
    std::memcpy(R, B.R.data(), B.R.size() * sizeof(double));
    return 0;
}
int orc_block_diffusion(void* h, int32_t b, const double* p, double* R) {
    Oracle* o = (Oracle*)h;
    orc::Block& B = o->blk[b];
    std::vector<double> pp(p, p + (size_t)o->nvar * o->ncell);
    std::fill(B.R.begin(), B.R.end(), 0.0);
    o->diffusion(B, pp);
    std::memcpy(R, B.R.data(), B.R.size() * sizeof(double));
    return 0;
}
// leaf (0-based block) owning a point given in the frame of panel `yin`, or -1
int orc_find_leaf(void* h, const double* rtp, int32_t yin) {
    const orc::Node* nd = ((Oracle*)h)->tree.find(rtp, yin != 0);
    return nd ? nd->leaf_id - 1 : -1;
}
// known-answer helpers
void orc_coord_conv(const double* in, double* out) { orc::coord_conv(in, out); }
void orc_vec_conv(const double* rtp, const double* v, double* out) { orc::vec_conv(rtp, v, out); }
int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // extern "C"
