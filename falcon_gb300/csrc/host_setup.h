// host_setup.h -- one-time host-side setup of the Yin-Yang block grid.
//
// Builds, on the host, everything the device step needs and that the reference
// builds once at start-up: the Yin-Yang block tree (3_6/ModYinYangTree.f90),
// per-block geometry (3_6/ModBlock.f90:288-438), the 1D background profiles
// (3_6/ModBlock.f90:188-265 fed by a get_vars-style provider) and the ghost map
// (3_6/ModGC.f90:25-147 + 3_6/ModCommunication.f90:219-366).
#pragma once
#include <cstdint>
#include <string>
#include <memory>
#include <utility>
#include <vector>

#include "../../include/falcon_gb300.h"

namespace falcon {

// Ideal-gas polytrope behind the get_vars interface
// (3_6/ModStratification_new.f90:352-384 signature).
struct Polytrope {
    double n, rb, rt, zeta_t, K, rho_b, g_b, p_b, R_gas, T_b, c_top;
    int xi_mode;
    void init(const falcon_background_spec& s, double r_lo, double r_hi);
    // g, rho0, p0, T0, gamma1, gamma3, diffusion, cooling, Xi
    void get_vars(double r, double* out) const;
    double middle_r(double r_lo, double r_hi) const;
};

// Flat Yin-Yang tree: node 0 is the Yin root, node 1 the Yang root; the
// children of a node are contiguous.
struct TreeNode {
    double rng[3][2];
    int32_t first_child = -1, nchild = 0, leaf = -1;
    uint8_t yin = 1;
};

struct GhostMapEntry {          // falcon_ghost_entry plus derived interpolation data
    falcon_ghost_entry e;
    int32_t i0, j0, k0;         // source base cell (Fortran indices)
    double w[3];
    uint8_t copy, rotate;
    double rot[2];              // sin(phi_s)*sin(phi_t), cos(phi_s)/sin(theta_t)
};

// std::allocator whose resize() leaves trivially constructible elements
// uninitialised: the ghost map (about 2 GB for a 21M-cell shell) is then
// written once, in parallel, instead of being zero-filled serially first
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = DefaultInitAlloc<U>; };
    DefaultInitAlloc() = default;
    template <class U> DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept {}
    template <class U> void construct(U* p) noexcept { ::new ((void*)p) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};

struct Grid {
    falcon_config cfg;
    int ni, nj, nk, ng, nip, njp, nkp, ncell;
    double r_range[2];
    Polytrope bg;
    std::vector<TreeNode> nodes;
    int nblocks = 0, nblocks_yin = 0;
    std::vector<int32_t> leaf_node;       // block -> node id
    std::vector<double> ranges;           // [b][3][2]
    std::vector<int32_t> flags;           // bit0 yin, bit1 top, bit2 bottom
    std::vector<double> xi, xj, xk;       // [b][nip], [b][njp], [b][nkp]
    std::vector<double> dx;               // [b][3]
    std::vector<double> prof;             // [b][FALCON_NPROF][nip]
    std::vector<GhostMapEntry, DefaultInitAlloc<GhostMapEntry>> ghosts;   // canonical (reference) order
    int64_t uncovered = 0;                // non-radial ghosts without owner

    // returns empty string on success, else the error message; with_ghosts=false
    // builds the tree, geometry and background only (the solvers' grids)
    std::string build(const falcon_config& c, bool with_ghosts = true);
    int find_leaf(const double* rtp, bool yin) const;
};

}  // namespace falcon
