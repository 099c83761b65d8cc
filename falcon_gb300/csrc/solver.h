// solver.h -- implicit solvers on the Yin-Yang block grid: the face-coefficient
// operator, its multigrid hierarchy and 1-layer halo maps (host side).
//
// Reference: 3_5/ModMultigrid.f90 (levels, geometry), 3_5/ModGC.f90:53-284 and
// 3_5/ModCommunication.f90:1497-1639 (1-layer face-ghost halo), 3_5/ModPFSS.f90
// (PFSS operator), 3_5/ModLinearSolver.f90 (SpMV, V-cycle, MG-CG).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "host_setup.h"

namespace falcon {

// One face ghost of level-l block `tb` filled by trilinear interpolation from
// the interior of block `sb` (same level): the form of ModMath_3D_interpolate_1D
// (3_5/ModMath.f90:208-248) with the base cell clamped to the source interior.
struct HaloEntry {
    int32_t tb, ti, tj, tk;      // target block and padded (0..m+1) cell
    int32_t sb, i0, j0, k0;      // source block and base interior cell (1..m-1 or m when weight 0)
    double w[3];
    double src_x[3];             // ghost centre in the source panel's frame
};

struct SolverLevel {
    int m[3] = {0, 0, 0};          // interior cells per block
    std::vector<double> xi, xj, xk;   // [b][m+2] cell centres incl. the ghost layer
    std::vector<double> dx;            // [b][3]
    // face-coefficient operator (3_5/ModBlock.f90:39-44):
    // Aii[b][k][j][i], Ai[b][k][j][i+1 faces], Aj[b][k][j faces][i], Ak[b][k faces][j][i]
    std::vector<double> Aii, Ai, Aj, Ak, V;
    std::vector<HaloEntry> halo;
    int nint() const { return m[0] * m[1] * m[2]; }
};

// A set of independent problems solved together (batched PFSS) or one problem
// (conduction): blocks of all problems are numbered consecutively.
struct SolverProblemSet {
    int nlevels = 0;
    int nproblems = 0;
    int nblocks = 0;
    std::vector<int32_t> block_problem;   // [b]
    std::vector<int32_t> block_flags;     // bit0 yin, bit1 top, bit2 bottom
    std::vector<int32_t> problem_first_block;  // [p+1]
    std::vector<SolverLevel> L;            // [level]
    std::vector<double> b;                 // right-hand side, level 0, [b][nint]
    std::vector<double> x0;                // initial guess, level 0
    std::vector<double> br;                // PFSS: Br at the bottom faces [b][k][j] (0 off the bottom blocks)
    std::vector<Grid> grids;               // one tree per problem
    std::string err;
};

// Face areas, distances and volumes of one block at one level
// (3_5/ModMultigrid.f90:97-233, iGeometry=1), FP64.
struct LevelGeometry {
    int m[3];
    std::vector<double> xiI, xjI, xkI, xiF, xjF, xkF;   // centres 0..m+1, faces 1..m+1
    double dxi, dxj, dxk;
    double Si(int i, int j, int k) const;   // i in 1..m+1
    double Sj(int i, int j, int k) const;
    double Sk(int i, int j, int k) const;
    double Di(int i, int j, int k) const;
    double Dj(int i, int j, int k) const;
    double Dk(int i, int j, int k) const;
    double Vol(int i, int j, int k) const;
    void init(const double rng[3][2], const int mm[3]);
};

// Build levels, halo maps and geometry for the problems' trees. The number of
// levels is capped by nlevels_max and by the largest power-of-two divisor
// depth of the block size (3_5/ModMultigrid.f90:76-88).
std::string build_solver_levels(SolverProblemSet& S, const std::vector<falcon_config>& cfgs, int nlevels_max);

// PFSS operator and right-hand side (3_5/ModPFSS.f90:21-100); magnetogram
// Br at the bottom faces of bottom blocks: br[b][k][j] per level-0 block (only
// bottom blocks read).
void assemble_pfss(SolverProblemSet& S, const std::vector<double>& br_bottom);
// Only the PFSS right-hand side from a bottom-face Br (the operator does not
// depend on it): S.b and S.br.
void pfss_rhs(SolverProblemSet& S, const std::vector<double>& br_bottom);

// Coarse operators A_c = P^T A P for levels 1.. from level 0 (P: injection).
void galerkin_coarsen(SolverProblemSet& S);

// Implicit anisotropic conduction operator (backward Euler) and right-hand side.
struct ConductionField;
void assemble_conduction(SolverProblemSet& S, const ConductionField& F, double dt_factor, double* dt_out);

// Synthetic temperature and magnetic field for the conduction workload.
struct ConductionField {
    const Polytrope* bg;
    double kappa0, floor_frac;
    double ell;                                   // correlation length of log T
    std::vector<double> kx, ky, kz, ph;           // Gaussian-field modes
    std::vector<double> qx, qy, qz, q;            // buried point charges
    void init(const Polytrope* b, uint64_t seed, double r_lo);
    double temperature(const double* xyz, double r) const;
    void bfield(const double* xyz, double* B) const;   // Yin-frame Cartesian
};

// Synthetic magnetogram for one problem: tilted bipoles + dipole (Yin frame).
struct Magnetogram {
    std::vector<double> px, py, pz, q;    // point charges just below the surface
    double dipole_g = 1.0;
    void init(uint64_t seed, double r_surface);
    double br(double r, double theta, double phi) const;   // Yin frame
};

}  // namespace falcon
