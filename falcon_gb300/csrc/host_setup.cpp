// host_setup.cpp -- Yin-Yang tree, block geometry, background and ghost map.
//
// Arithmetic follows the reference operation by operation (the maps must be
// bit-identical to the reference's), while the data structures are built for
// a one-GPU consumer: a flat node array instead of a pointer tree, each ghost
// point converted to both panel frames once instead of per node test, and the
// per-block map build parallelised over blocks.
//
// Default-real (FP32) literals of the Fortran are reproduced as float values
// promoted to double (gfortran semantics).
#include "host_setup.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>

namespace falcon {

static const float kPiF = 3.1415926535f;                  // 3_6/ModConst.f90:2 (real)
static const double kRsun = (double)6.955e10f;            // 3_6/ModConst.f90:5
static const double kKB = (double)1.380649e-16f;          // 3_6/ModConst.f90:9
static const double kMp = (double)1.67262192369e-24f;     // 3_6/ModConst.f90:10
static const double kGamma = (double)(5.0f / 3.0f);       // 3_6/ModConst.f90:12

// ---- background -----------------------------------------------------------
void Polytrope::init(const falcon_background_spec& s, double r_lo, double r_hi) {
    n = s.poly_n;
    xi_mode = s.xi_mode;
    rb = r_lo;
    rt = r_hi;
    zeta_t = std::pow(s.density_contrast, -1.0 / n);
    K = (1.0 - zeta_t) / (1.0 / rb - 1.0 / rt);
    rho_b = std::pow(10.0, -0.6841807359334023);   // base density, 3_6/ModStratification_new.f90:29
    g_b = 54340.03688603464;                       // base gravity, 3_6/ModStratification_new.f90:30
    p_b = rho_b * g_b * rb * rb / ((n + 1.0) * K);
    R_gas = kKB / (s.mu * kMp);
    T_b = p_b / (rho_b * R_gas);
    double zt = 1.0 + K * (1.0 / rt - 1.0 / rb);
    double rho_t = rho_b * std::pow(zt, n);
    double p_t = p_b * std::pow(zt, n + 1.0);
    c_top = std::sqrt(kGamma * p_t / rho_t);
}

void Polytrope::get_vars(double r, double* o) const {
    double z = 1.0 + K * (1.0 / r - 1.0 / rb);
    double q = rb / r;
    o[0] = g_b * (q * q);
    o[1] = rho_b * std::pow(z, n);
    o[2] = p_b * std::pow(z, n + 1.0);
    o[3] = T_b * z;
    o[4] = kGamma;
    o[5] = kGamma;
    o[6] = 0.0;   // radiative heating: 0 for the polytrope
    o[7] = 0.0;   // artificial cooling: 0
    o[8] = xi_mode ? std::sqrt(o[4] * o[2] / o[1]) / c_top : 1.0;
}

// Radius that bisects the integral of |d ln rho0/dr| over [r_lo, r_hi]
// (3_6/ModStratification_new.f90:388-432, 200 uniform samples, trapezoid rule).
double Polytrope::middle_r(double r_lo, double r_hi) const {
    constexpr int m = 200;
    const double dr = (r_hi - r_lo) / (double)m;
    double rho[m + 1], f[m + 1], acc[m + 1], o[FALCON_NPROF];
    for (int s = 0; s <= m; ++s) {
        get_vars(r_lo + s * dr, o);
        rho[s] = o[1];
    }
    f[0] = std::fabs(rho[1] - rho[0]) / (dr * rho[0]);
    f[m] = std::fabs(rho[m] - rho[m - 1]) / (dr * rho[m]);
    for (int s = 1; s < m; ++s) f[s] = std::fabs(rho[s + 1] - rho[s - 1]) / (2.0 * dr * rho[s]);
    acc[0] = 0.0;
    for (int s = 1; s <= m; ++s) acc[s] = acc[s - 1] + 0.5 * (f[s] + f[s - 1]) * dr;
    const double half = 0.5 * acc[m];
    for (int s = 1; s <= m; ++s)
        if (acc[s] >= half) return (r_lo + (s - 1) * dr) + (half - acc[s - 1]) / (acc[s] - acc[s - 1]) * dr;
    return r_hi;
}

// ---- Yin-Yang coordinate transform (3_6/ModYinYang.f90:8-17) -------------
static inline void yy_convert(const double* a, double* b) {
    const double st = std::sin(a[1]), ct = std::cos(a[1]);
    const double sp = std::sin(a[2]), cp = std::cos(a[2]);
    b[0] = a[0];
    b[1] = std::acos(st * sp);
    const double den = std::sqrt(st * st * (cp * cp) + ct * ct);
    b[2] = std::copysign(std::fabs(std::acos(-(st * cp) / den)), ct);
}

// ---- tree construction -----------------------------------------------------
namespace {

struct Builder {
    std::vector<TreeNode>& nodes;
    const Polytrope& bg;

    // N-way split with the YinYangTree_Divide formula (3_6/ModYinYangTree.f90:239-264)
    void split(int id, const int N[3]) {
        if (nodes[id].nchild != 0) return;
        const int first = (int)nodes.size();
        nodes.resize(nodes.size() + (size_t)N[0] * N[1] * N[2]);
        const TreeNode p = nodes[id];
        int c = first;
        for (int ir = 1; ir <= N[0]; ++ir) {
            const double lo_e = (double)(((float)(N[0] - ir) + 1.0f) / (float)N[0]);
            const double hi_e = (double)(((float)(N[0] - ir) + 0.0f) / (float)N[0]);
            const double lo_d = (double)(((float)(-ir) + 1.0f) / (float)N[0]);
            const double hi_d = (double)(((float)(-ir) + 0.0f) / (float)N[0]);
            const double rlo = std::pow(p.rng[0][0], lo_e) / std::pow(p.rng[0][1], lo_d);
            const double rhi = std::pow(p.rng[0][0], hi_e) / std::pow(p.rng[0][1], hi_d);
            for (int it = 1; it <= N[1]; ++it) {
                const double tlo = p.rng[1][0] * (double)((float)(N[1] - it) + 1.0f) / (double)N[1] -
                                   p.rng[1][1] * (double)((float)(-it) + 1.0f) / (double)N[1];
                const double thi = p.rng[1][0] * (double)((float)(N[1] - it) + 0.0f) / (double)N[1] -
                                   p.rng[1][1] * (double)((float)(-it) + 0.0f) / (double)N[1];
                for (int ip = 1; ip <= N[2]; ++ip) {
                    TreeNode& ch = nodes[c++];
                    ch.yin = p.yin;
                    ch.rng[0][0] = rlo; ch.rng[0][1] = rhi;
                    ch.rng[1][0] = tlo; ch.rng[1][1] = thi;
                    ch.rng[2][0] = p.rng[2][0] * (double)((float)(N[2] - ip) + 1.0f) / (double)N[2] -
                                   p.rng[2][1] * (double)((float)(-ip) + 1.0f) / (double)N[2];
                    ch.rng[2][1] = p.rng[2][0] * (double)((float)(N[2] - ip) + 0.0f) / (double)N[2] -
                                   p.rng[2][1] * (double)((float)(-ip) + 0.0f) / (double)N[2];
                }
            }
        }
        nodes[id].first_child = first;
        nodes[id].nchild = N[0] * N[1] * N[2];
    }

    // two radial children (3_6/ModYinYangTree.f90:158-206)
    void split_r(int id, int option) {
        if (nodes[id].nchild != 0) return;
        const TreeNode p = nodes[id];
        double mid = 0.0;
        if (option == 1) mid = bg.middle_r(p.rng[0][0], p.rng[0][1]);
        else if (option == 2) mid = (p.rng[0][0] + p.rng[0][1]) * 0.5;
        else if (option == 3) mid = std::sqrt(p.rng[0][0] * p.rng[0][1]);
        const int first = (int)nodes.size();
        nodes.resize(nodes.size() + 2);
        nodes[first] = p;
        nodes[first + 1] = p;
        nodes[first].first_child = nodes[first + 1].first_child = -1;
        nodes[first].nchild = nodes[first + 1].nchild = 0;
        nodes[first].rng[0][1] = mid;
        nodes[first + 1].rng[0][0] = mid;
        nodes[id].first_child = first;
        nodes[id].nchild = 2;
    }

    // visit the current leaves of a subtree in depth-first order
    void leaves_of(int id, std::vector<int>& out) const {
        if (nodes[id].nchild == 0) { out.push_back(id); return; }
        for (int c = 0; c < nodes[id].nchild; ++c) leaves_of(nodes[id].first_child + c, out);
    }
};

// 3_6/ModMath.f90:5-16
bool open_overlap(const double* a, const double* b) {
    return (a[0] - b[0]) * (a[0] - b[1]) < 0.0 || (a[1] - b[0]) * (a[1] - b[1]) < 0.0 ||
           (b[0] - a[0]) * (b[0] - a[1]) < 0.0 || (b[1] - a[0]) * (b[1] - a[1]) < 0.0;
}

}  // namespace

// closed-interval containment of a point already expressed in the node's frame
static inline bool contains(const TreeNode& n, const double* h) {
    return (h[0] - n.rng[0][0]) * (h[0] - n.rng[0][1]) <= 0.0 &&
           (h[1] - n.rng[1][0]) * (h[1] - n.rng[1][1]) <= 0.0 &&
           (h[2] - n.rng[2][0]) * (h[2] - n.rng[2][1]) <= 0.0;
}

// Depth-first first match with backtracking, semantics of
// YinYangTree_FindNode / _OneBranch (3_6/ModYinYangTree.f90:449-505).
// p[0]: the point in the Yin frame, p[1]: in the Yang frame.
static int find_in(const std::vector<TreeNode>& nodes, int id, const double (*p)[3]) {
    const TreeNode& n = nodes[id];
    const double* h = p[n.yin ? 0 : 1];
    if (!contains(n, h)) return -1;
    if (n.nchild == 0) return n.leaf;
    for (int c = 0; c < n.nchild; ++c) {
        const int cid = n.first_child + c;
        if (!contains(nodes[cid], h)) continue;
        const int r = find_in(nodes, cid, p);
        if (r >= 0) return r;
    }
    return -1;
}

int Grid::find_leaf(const double* rtp, bool yin) const {
    double p[2][3];
    const int own = yin ? 0 : 1;
    std::memcpy(p[own], rtp, 3 * sizeof(double));
    yy_convert(rtp, p[1 - own]);
    const int root = contains(nodes[0], p[0]) ? 0 : 1;
    return find_in(nodes, root, p);
}

std::string Grid::build(const falcon_config& c, bool with_ghosts) {
    cfg = c;
    const falcon_tree_spec& t = c.tree;
    if (t.ni < 4 || t.nj < 4 || t.nk < 4 || t.ng != 2)
        return "block sizes must be >= 4 and ng must be 2 (fourth-order stencils)";
    (void)with_ghosts;
    if (t.ni > 32 || t.nj > 32 || t.nk > 32) return "block sizes above 32 are not supported";
    if (c.phys.divb_option < 0 || c.phys.divb_option > 2)
        return "divb_option must be 0 (none), 1 (GLM) or 2 (Powell source term)";
    if (c.phys.divb_option != 0 && !c.phys.if_involve_B) return "divb_option 1 or 2 needs if_involve_B = 1";
    if (with_ghosts && !c.phys.if_involve_B) return "if_involve_B must be 1 (the MHD block layout with B active)";
    if (t.radial_option < 1 || t.radial_option > 3) return "radial_option must be 1, 2 or 3";
    if (t.n_amr < 0 || t.n_amr > FALCON_MAX_AMR) return "n_amr out of range";
    for (int d = 0; d < 3; ++d)
        if (t.root_tiles[d] < 1) return "root_tiles must be >= 1";
    ni = t.ni; nj = t.nj; nk = t.nk; ng = t.ng;
    nip = ni + 2 * ng; njp = nj + 2 * ng; nkp = nk + 2 * ng;
    ncell = nip * njp * nkp;
    r_range[0] = t.r_range_rsun[0] * kRsun;    // 3_6/ModReadParameters.f90:71
    r_range[1] = t.r_range_rsun[1] * kRsun;
    bg.init(c.bg, r_range[0], r_range[1]);

    // roots: theta in [pi/4, 3pi/4], phi in [-3pi/4, 3pi/4], FP32 products
    nodes.clear();
    nodes.resize(2);
    for (int k = 0; k < 2; ++k) {
        TreeNode& r = nodes[k];
        r.yin = (k == 0);
        r.rng[0][0] = r_range[0]; r.rng[0][1] = r_range[1];
        r.rng[1][0] = (double)(kPiF * 0.25f); r.rng[1][1] = (double)(kPiF * 0.75f);
        r.rng[2][0] = (double)(-(kPiF * 0.75f)); r.rng[2][1] = (double)(kPiF * 0.75f);
    }
    Builder bld{nodes, bg};
    if ((int64_t)t.root_tiles[0] * t.root_tiles[1] * t.root_tiles[2] > 1) {
        bld.split(0, t.root_tiles);
        bld.split(1, t.root_tiles);
    }
    std::vector<int> lv;
    for (int l = 0; l < t.radial_levels; ++l)
        for (int root = 0; root < 2; ++root) {
            lv.clear();
            bld.leaves_of(root, lv);
            for (int id : lv) bld.split_r(id, t.radial_option);
        }
    for (int l = 0; l < t.n_amr; ++l) {
        const int N[3] = {t.amr_divide[l][0] ? 2 : 1, t.amr_divide[l][1] ? 2 : 1, t.amr_divide[l][2] ? 2 : 1};
        const double rr[2] = {t.amr_range[l][0][0] * kRsun, t.amr_range[l][0][1] * kRsun};
        for (int root = 0; root < 2; ++root) {
            lv.clear();
            bld.leaves_of(root, lv);
            for (int id : lv) {
                const TreeNode& n = nodes[id];
                bool hit;
                if (t.amr_global[l]) hit = open_overlap(n.rng[0], rr);
                else hit = n.yin && open_overlap(n.rng[0], rr) && open_overlap(n.rng[1], t.amr_range[l][1]) &&
                           open_overlap(n.rng[2], t.amr_range[l][2]);
                if (hit) bld.split(id, N);
            }
        }
    }
    // leaf numbering: Yin depth-first, then Yang (3_6/ModYinYangTree.f90:402-420)
    leaf_node.clear();
    lv.clear(); bld.leaves_of(0, lv);
    nblocks_yin = (int)lv.size();
    bld.leaves_of(1, lv);
    nblocks = (int)lv.size();
    if (nblocks > (1 << 20)) return "too many blocks";
    leaf_node = lv;
    for (int b = 0; b < nblocks; ++b) nodes[lv[b]].leaf = b;

    // geometry (3_6/ModBlock.f90:288-438) and background (3_6/ModBlock.f90:188-265)
    ranges.assign((size_t)nblocks * 6, 0.0);
    flags.assign(nblocks, 0);
    xi.assign((size_t)nblocks * nip, 0.0);
    xj.assign((size_t)nblocks * njp, 0.0);
    xk.assign((size_t)nblocks * nkp, 0.0);
    dx.assign((size_t)nblocks * 3, 0.0);
    prof.assign((size_t)nblocks * FALCON_NPROF * nip, 0.0);
    auto centres = [](const double* rg, int n, int g, double* out) {
        for (int i = 1 - g; i <= n + g; ++i)
            out[i + g - 1] = (rg[0] * (double)((float)(n - i) + 0.5f) + rg[1] * (double)((float)i - 0.5f)) / n;
    };
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nblocks; ++b) {
        const TreeNode& n = nodes[leaf_node[b]];
        std::memcpy(&ranges[(size_t)b * 6], n.rng, 6 * sizeof(double));
        centres(n.rng[0], ni, ng, &xi[(size_t)b * nip]);
        centres(n.rng[1], nj, ng, &xj[(size_t)b * njp]);
        centres(n.rng[2], nk, ng, &xk[(size_t)b * nkp]);
        dx[3 * b + 0] = (n.rng[0][1] - n.rng[0][0]) / ni;
        dx[3 * b + 1] = (n.rng[1][1] - n.rng[1][0]) / nj;
        dx[3 * b + 2] = (n.rng[2][1] - n.rng[2][0]) / nk;
        int f = n.yin ? 1 : 0;
        if (xi[(size_t)b * nip + nip - 1] > r_range[1]) f |= 2;   // 3_6/ModYinYangTree.f90:273-288
        if (xi[(size_t)b * nip] < r_range[0]) f |= 4;
        flags[b] = f;
        double o[FALCON_NPROF];
        for (int i = 0; i < nip; ++i) {
            bg.get_vars(xi[(size_t)b * nip + i], o);
            for (int p = 0; p < FALCON_NPROF; ++p) prof[((size_t)b * FALCON_NPROF + p) * nip + i] = o[p];
        }
    }

    if (!with_ghosts) return "";
    // ghost map: owners in i-j-k loop order (k fastest), grouped per source leaf
    // in first-appearance order (3_6/ModGC.f90:25-147)
    std::vector<std::vector<GhostMapEntry>> per(nblocks);
    int64_t unc = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : unc)
    for (int b = 0; b < nblocks; ++b) {
        const bool yin = flags[b] & 1;
        const double* X = &xi[(size_t)b * nip];
        const double* Y = &xj[(size_t)b * njp];
        const double* Z = &xk[(size_t)b * nkp];
        std::vector<int32_t> owner;
        std::vector<int32_t> cell;
        owner.reserve(ncell); cell.reserve(ncell);
        for (int i = 1 - ng; i <= ni + ng; ++i)
            for (int j = 1 - ng; j <= nj + ng; ++j)
                for (int k = 1 - ng; k <= nk + ng; ++k) {
                    if (i >= 1 && i <= ni && j >= 1 && j <= nj && k >= 1 && k <= nk) continue;
                    const double rtp[3] = {X[i + ng - 1], Y[j + ng - 1], Z[k + ng - 1]};
                    const int o = find_leaf(rtp, yin);
                    if (o < 0) {
                        if (rtp[0] > r_range[0] && rtp[0] < r_range[1]) ++unc;
                        continue;
                    }
                    owner.push_back(o);
                    cell.push_back(((i + ng - 1) * 64 + (j + ng - 1)) * 64 + (k + ng - 1));
                }
        // stable grouping by first appearance of the owner: rank the owners in
        // first-appearance order, then bucket the entries by rank (linear)
        std::vector<int32_t> seen, rank(owner.size());
        for (size_t q = 0; q < owner.size(); ++q) {
            const auto it = std::find(seen.begin(), seen.end(), owner[q]);
            rank[q] = (int32_t)(it - seen.begin());
            if (it == seen.end()) seen.push_back(owner[q]);
        }
        std::vector<int32_t> start(seen.size() + 1, 0), order(owner.size());
        for (size_t q = 0; q < owner.size(); ++q) ++start[rank[q] + 1];
        for (size_t r = 0; r < seen.size(); ++r) start[r + 1] += start[r];
        {
            std::vector<int32_t> fill(start.begin(), start.end() - 1);
            for (size_t q = 0; q < owner.size(); ++q) order[fill[rank[q]]++] = (int32_t)q;
        }
        auto& out = per[b];
        out.reserve(owner.size());
        for (size_t r = 0; r < seen.size(); ++r) {
            const int32_t s = seen[r];
            const bool syin = flags[s] & 1;
            const double* SX = &xi[(size_t)s * nip];
            const double* SY = &xj[(size_t)s * njp];
            const double* SZ = &xk[(size_t)s * nkp];
            // ModMath_1D3D_interpolate_1D1D set-up (3_6/ModMath.f90:264-281)
            // spacing x(2)-x(1) from the coordinate array; Fortran index i sits at i+ng-1
            const double sdx[3] = {SX[ng + 1] - SX[ng], SY[ng + 1] - SY[ng], SZ[ng + 1] - SZ[ng]};
            const double s0[3] = {SX[0], SY[0], SZ[0]};
            const double nmax[3] = {(double)((float)ni + 0.0f), (double)((float)nj + 0.0f), (double)((float)nk + 0.0f)};
            const double off = (double)((float)(-ng) + 1.0f);
            for (int32_t oq = start[r]; oq < start[r + 1]; ++oq) {
                const size_t q = (size_t)order[oq];
                const int i = cell[q] / 4096 - ng + 1, j = (cell[q] / 64) % 64 - ng + 1, k = cell[q] % 64 - ng + 1;
                GhostMapEntry g{};
                g.e.tblock = b; g.e.ti = i; g.e.tj = j; g.e.tk = k;
                g.e.sblock = s;
                const double x[3] = {X[i + ng - 1], Y[j + ng - 1], Z[k + ng - 1]};
                if (syin == yin) std::memcpy(g.e.src_x, x, sizeof(x));
                else yy_convert(x, g.e.src_x);
                int base[3];
                for (int d = 0; d < 3; ++d) {
                    double p = off + (g.e.src_x[d] - s0[d]) / sdx[d];
                    p = std::max(std::min(p, nmax[d]), 1.0);
                    base[d] = (int)std::floor(p);
                    g.w[d] = p - base[d];
                }
                g.i0 = base[0]; g.j0 = base[1]; g.k0 = base[2];
                g.copy = (g.w[0] == 0.0 && g.w[1] == 0.0 && g.w[2] == 0.0);
                g.rotate = (syin != yin);
                if (g.rotate) {
                    // ModYinYang_VecConv coefficients at the source-frame point (3_6/ModYinYang.f90:48-61)
                    double back[3];
                    yy_convert(g.e.src_x, back);
                    g.rot[0] = std::sin(g.e.src_x[2]) * std::sin(back[2]);
                    g.rot[1] = std::cos(g.e.src_x[2]) / std::sin(back[1]);
                }
                out.push_back(g);
            }
        }
    }
    uncovered = unc;
    // concatenate in block order, in parallel (the map of a 21M-cell shell is
    // about 2 GB)
    std::vector<size_t> offs((size_t)nblocks + 1, 0);
    for (int b = 0; b < nblocks; ++b) offs[b + 1] = offs[b] + per[b].size();
    ghosts.clear();
    ghosts.resize(offs[nblocks]);
#pragma omp parallel for schedule(dynamic, 16)
    for (int b = 0; b < nblocks; ++b) {
        std::copy(per[b].begin(), per[b].end(), ghosts.begin() + (long)offs[b]);
        std::vector<GhostMapEntry>().swap(per[b]);
    }
    if (uncovered > 0) return "ghost cells inside the radial range have no owner leaf";
    return "";
}

}  // namespace falcon
