/*
 * falcon_gb300.h -- C ABI of the GB300-native Falcon hot path.
 *
 * Plain C: fixed-width integers, doubles, opaque handles. No C++ or torch
 * types cross this boundary, so an iso_c_binding shim (Fortran), ctypes
 * (Python) or any C caller binds it directly.
 *
 * Conventions
 *   - Every entry point returns int: FALCON_OK (0) or a negative FALCON_ERR_*.
 *     No exception or longjmp crosses the ABI. falcon_last_error() returns the
 *     message of the most recent failure on a context.
 *   - The library owns all device memory. Host pointers are borrowed for the
 *     duration of a call only.
 *   - One host thread per context; a context is not re-entrant. All device work
 *     of a context runs on one CUDA stream owned by the context.
 *   - Block arrays use the reference's Fortran layout: primitive(i,j,k,var)
 *     with bounds (-ng+1:ni+ng, -ng+1:nj+ng, -ng+1:nk+ng, 1:nvar), i fastest
 *     (3_6/ModBlock.f90:275-277). Variables are rho1, vr, vt, vp, br, bt, bp, s1,
 *     psi (3_6/ModBlock.f90:153-163): FALCON_NVAR = 9, as the reference's MHD
 *     block. psi is evolved only with divb_option = 1 (GLM cleaning); with 0 it
 *     is not stored on the device, must be 0 on upload and downloads as 0,
 *     which is what the reference keeps for a psi that starts at 0.
 *
 * The entry points replace these reference interfaces:
 *   falcon_create ........... YinYangTree_InitTree/ModAMR_set_grid/YinYangTree_SetAll
 *                             (3_6/test1.f90:110-120) and ModCommunication_SetGCAll
 *                             (3_6/ModCommunication.f90:22-64)
 *   falcon_upload_state ..... writes Tree%LocalBlocks(:)%primitive_IV (3_6/ModBlock.f90:62)
 *   falcon_download_state ... reads it back (for ModSave_DoAll / ModCheck)
 *   falcon_exchange ......... ModCommunication_SendRecvGC_new(Tree,.false.)
 *                             (3_6/ModCommunication.f90:655-795)
 *   falcon_timestep ......... ModWaveSpeed_Dynamo + ModTimeStep_Dynamo + MPI MIN
 *                             (3_6/ModWaveSpeed.f90:8-27, 3_6/ModTimeStep.f90:10-30,
 *                             3_6/ModAdvance.f90:31-48)
 *   falcon_step_rk4 ......... ModAdvance_rk4 (3_6/ModAdvance.f90:18-112)
 *   falcon_set_background ... ModBlock_InitSSM's profiles from ModStratification_new_get_vars
 *                             (3_6/ModBlock.f90:233-264)
 */
#ifndef FALCON_GB300_H
#define FALCON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define FALCON_OK                    0
#define FALCON_ERR_INVALID_ARG      -1
#define FALCON_ERR_CUDA             -2
#define FALCON_ERR_NAN_DETECTED     -3  /* replaces MPI_Abort in 3_6/ModCheck.f90:38,61 */
#define FALCON_ERR_TIMEOUT          -4
#define FALCON_ERR_NOT_CONVERGED    -5
#define FALCON_ERR_BOUNDS           -6
#define FALCON_ERR_UNCOVERED_GHOST  -7  /* a non-radial ghost cell has no owner leaf */
#define FALCON_ERR_NO_DEVICE        -8

/* ---- precision modes ---------------------------------------------------- */
/* FP64: every operation in IEEE double, no FMA contraction, same operation
 *       order as the reference; bit-comparable with the CPU oracle.
 * MIXED: state stored in FP32, u^n with an 8-bit correction of its FP32
 *       rounding that the end-of-step updates carry (error-free FP32 sums);
 *       stencil RHS and stage updates in FP32; the linearised-EOS pressure p1
 *       (where the background terms nearly cancel) is assembled in float-float
 *       (exact FP32 products with the coefficients' (hi, lo) FP32 pairs and an
 *       error-free sum, about as accurate as an FP64 assembly, with no FP64
 *       instruction per cell); the per-cell CFL ratio h/v_wave is formed in
 *       explicitly rounded FP32, each block's minimum is widened to FP64 for
 *       the cross-block min-reduction (an atomic on FP64 bits), and dt =
 *       CFL * min is FP64. */
#define FALCON_PREC_FP64   0
#define FALCON_PREC_MIXED  1

#define FALCON_MAX_AMR 16
#define FALCON_NVAR 9
/* number of 1D radial background profiles per block (see falcon_get_background) */
#define FALCON_NPROF 9

/* Grid/tree description: the values PARAM.in carries in #DOMAIN, #GRID,
 * #RADIALGRID and #AMR (3_6/ModReadParameters.f90:60-106,408-483), plus a root
 * tiling. root_tiles = {1,1,1} is the reference tree exactly; other values split
 * each panel root once into root_tiles[0] x [1] x [2] children with the same
 * formula YinYangTree_Divide uses for 2-way splits (3_6/ModYinYangTree.f90:245-255). */
typedef struct falcon_tree_spec {
    int32_t ni, nj, nk, ng;          /* cells per block, ghost layers */
    int32_t root_tiles[3];           /* root tiling per panel (r, theta, phi) */
    int32_t radial_levels;           /* #RADIALGRID rLevelInitial */
    int32_t radial_option;           /* YinYangTree_Divide_r i_option (1,2,3) */
    int32_t n_amr;                   /* #AMR nAMRs */
    int32_t amr_divide[FALCON_MAX_AMR][3];   /* rtp_if_divide per AMR level */
    int32_t amr_global[FALCON_MAX_AMR];      /* if_global */
    double  amr_range[FALCON_MAX_AMR][3][2]; /* r in R_sun; theta, phi in rad */
    double  r_range_rsun[2];         /* #DOMAIN r_range (R_sun) */
} falcon_tree_spec;

/* Physics switches of the Dynamo equations (3_6/ModEquation.f90:24-37). */
typedef struct falcon_physics {
    int32_t if_involve_B;            /* iEquation=1 with if_involve_B */
    int32_t divb_option;             /* DivB_option: 0 none; 1 GLM cleaning (3_6/ModDivB.f90:13-38);
                                        2 Powell source term -(div B) v (3_5/ModEquation.f90:169-176;
                                        3_6 declares 2 as Powell's term, ModParameters.f90:70, but its
                                        ModAdvance applies only 1, so a 3_6 run with 2 steps as 0) */
    double  cfl;                     /* #TIMESTEPPING CFL */
    double  heating_ratio;           /* Artificial_heating_ratio */
} falcon_physics;

/* Synthetic background: an ideal-gas polytrope served through the same 1D
 * profile interface as ModStratification_new_get_vars
 * (3_6/ModStratification_new.f90:352-384). */
typedef struct falcon_background_spec {
    double  poly_n;                  /* polytropic index (1.5) */
    double  density_contrast;        /* rho0(r_bottom)/rho0(r_top) (100) */
    double  mu;                      /* mean molecular weight for T0 */
    int32_t xi_mode;                 /* 0: Xi=1; 1: Xi=c_s/c_s(r_top) as ModStratification_new_calc_Xi */
    int32_t pad_;
} falcon_background_spec;

typedef struct falcon_config {
    falcon_tree_spec       tree;
    falcon_physics         phys;
    falcon_background_spec bg;
    int32_t                precision; /* FALCON_PREC_* */
    int32_t                device;    /* CUDA device ordinal */
} falcon_config;

typedef struct falcon_ctx falcon_ctx;

/* One ghost-map entry: how ghost cell (ti,tj,tk) of block tblock is filled.
 * Reference counterpart: one element of GC_source%ijk_list/xijk_list
 * (3_6/ModBlock.f90:7-15, filled by 3_6/ModGC.f90:53-147 and
 * 3_6/ModCommunication.f90:219-366). src_x are the ghost cell-centre
 * coordinates converted to the source block's panel frame. Block ids are
 * 0-based leaf numbers (iLeafNode-1); cell indices are the Fortran ones. */
typedef struct falcon_ghost_entry {
    int32_t tblock, ti, tj, tk;
    int32_t sblock, pad_;
    double  src_x[3];
} falcon_ghost_entry;

/* ---- lifetime ----------------------------------------------------------- */
/* Builds the Yin-Yang tree, the block geometry, the background and the ghost
 * map on the host, then allocates device state (unless device < 0, which
 * builds the host side only: enough for the map and geometry queries). */
int  falcon_create(falcon_ctx** out, const falcon_config* cfg);
void falcon_destroy(falcon_ctx* ctx);
int  falcon_last_error(const falcon_ctx* ctx, char* buf, size_t len);

/* ---- host-side geometry and map queries (no GPU needed) --------------- */
int  falcon_num_blocks(const falcon_ctx* ctx, int32_t* nblocks, int32_t* nblocks_yin);
/* ranges[b][3][2] of each leaf block (rtp_range, 3_6/ModYinYangTree.f90:24) */
int  falcon_block_ranges(const falcon_ctx* ctx, double* ranges);
/* flags[b] = bit0 if_yin, bit1 if_top, bit2 if_bottom */
int  falcon_block_flags(const falcon_ctx* ctx, int32_t* flags);
/* prof[b][FALCON_NPROF][ni+2ng]: g, rho0, p0, T0, gamma1, gamma3, diffusion,
 * cooling, Xi -- the outputs of ModStratification_new_get_vars at the cell
 * centres (3_6/ModBlock.f90:232-249) */
int  falcon_get_background(const falcon_ctx* ctx, double* prof);
/* Replace the background with the driver's own radial profiles, same layout
 * as falcon_get_background: prof[b][FALCON_NPROF][ni+2ng] = g, rho0, p0, T0,
 * gamma1, gamma3, diffusion, cooling, Xi at every block's cell centres (ghost
 * layers included) -- what ModBlock_InitSSM stores from
 * ModStratification_new_get_vars (3_6/ModBlock.f90:233-264,
 * 3_6/ModStratification_new.f90:352-384), e.g. from the FreeEOS/opacity
 * tables this library does not read. The device tables of every step kernel
 * are rebuilt from them (the GPU keeps 1-D profiles only). Rejected with
 * FALCON_ERR_INVALID_ARG, background unchanged, unless every value is finite
 * and rho0, p0, T0, gamma1 and Xi are positive. The next step re-forms the
 * CFL minimum. Valid on host-only contexts too (device < 0). */
int  falcon_set_background(falcon_ctx* ctx, const double* prof);
int  falcon_ghost_count(const falcon_ctx* ctx, int64_t* n);
/* entries in the reference's order: target block ascending, then its
 * GC_targets (first-appearance order of source leaves), then i-j-k loop order */
int  falcon_ghost_map(const falcon_ctx* ctx, falcon_ghost_entry* out, int64_t cap);

/* ---- state transfer (host pointers; blocking on the context stream) ---- */
/* u: nblocks x (Fortran block array incl. ghosts), FP64. In MIXED mode the
 * FP64<->FP32 conversion runs on the GPU through a device staging buffer. */
int  falcon_upload_state(falcon_ctx* ctx, const double* u);
int  falcon_download_state(falcon_ctx* ctx, double* u);
/* Download elements [first, first + count) of the falcon_download_state
 * layout into u (FP64), allocating nothing on the device or the host. It has
 * no counterpart in the reference, whose state is resident in host memory.
 *
 * Who needs it: in MIXED mode falcon_download_state stages through an FP64
 * device buffer of the whole host array (2.25x the FP32 state), allocated on
 * its first call. A caller whose state fills most of HBM has no room for that
 * buffer, and a caller that fixes its device footprint before the run (a
 * memory pool sized at start-up, a job that must not let a library grow its
 * memory mid-run, where cudaMalloc/cudaFree would also synchronise the whole
 * device) cannot let it be allocated. This call stages through one static
 * device array of FALCON_STATIC_SCRATCH_BYTES (16 MiB) compiled into the
 * library instead, so count is limited to FALCON_STATIC_SCRATCH_BYTES / 8
 * elements; larger counts, or a range past the end of the state, return
 * FALCON_ERR_INVALID_ARG without touching u. Download a whole state as a
 * sequence of ranges; ranges count elements of the host layout
 * ([block][FALCON_NVAR][cell]), gathered from the device state on the GPU.
 *
 * The first call on each device sets up the array's address
 * (cudaGetSymbolAddress; it may load the library's device code): make that
 * first call before any stream capture on the device. The address is cached
 * per device for the life of the process, which assumes that the device's
 * primary context is never reset (no cudaDeviceReset) while the library is
 * in use. Every context on a
 * device shares the one array, which keeps the last call's data; each call
 * synchronises the context stream before returning, but calls that overlap on
 * the GPU (from several host threads) race on the array: serialise them. */
#define FALCON_STATIC_SCRATCH_BYTES (16u << 20)
int  falcon_download_state_range(falcon_ctx* ctx, size_t first, size_t count, double* u);
/* Core transfers, for a driver that keeps the state on the host and moves it
 * every step: of every block and variable, only the interior planes and,
 * within them, the interior rows (whole, radial ghost columns included) move,
 * 64% of a 16^3 block's padded cells. falcon_upload_state_core recomputes the
 * theta/phi ghost layers on the device (the values the reference's
 * ModCommunication_SendRecvGC leaves there; the few ghost cells outside every
 * exchange list, the radial boundary columns of ghost rows, read as 0 until a
 * step's boundary condition rewrites them), forms the next step's CFL minimum,
 * and rejects a non-zero psi without GLM, leaving the state unchanged; any
 * earlier content of the device buffers (NaNs included) has no effect on the
 * uploaded state or the steps that follow; falcon_download_state_core
 * leaves the array's other cells untouched. Same array layout as
 * falcon_upload_state. The array must lie in a falcon_pin_host buffer and be
 * 16-byte aligned; otherwise, and for a core upload into an FP64 context, the
 * full transfer runs instead. Each run of interior rows starts on a 64-byte
 * line when the array does (16^3 blocks): a 64-byte-aligned array moves whole
 * lines over the host link, while the 16-mod-64 address of a large malloc
 * leaves partial lines at both ends of every run (the 21M-cell core download:
 * 188 against 175 GB/s). */
int  falcon_upload_state_core(falcon_ctx* ctx, const double* u);
int  falcon_download_state_core(falcon_ctx* ctx, double* u);
/* Page-lock a host buffer (cudaHostRegister, mapped) and remember it: a MIXED
 * falcon_upload_state / falcon_download_state whose whole array lies in such
 * a buffer converts straight from / into host memory on the GPU over the host
 * link (NVLink-C2C on GB300), with no device staging copy. Unpin before
 * freeing the buffer. */
int  falcon_pin_host(falcon_ctx* ctx, void* p, size_t bytes);
int  falcon_unpin_host(falcon_ctx* ctx, void* p);
/* synthetic initial condition generated on the device (seeded):
 * kind 0: Gaussian entropy bump + dipole B (v = 0)
 * kind 1: kind 0 plus a random-phase Kolmogorov velocity field (rms Mach mach) */
int  falcon_init_synthetic(falcon_ctx* ctx, int32_t kind, uint64_t seed, double mach);

/* ---- output and restart ------------------------------------------------- */
/* AllCells plot output from the device state, replacing ModSave_AllCells
 * (3_6/ModSavePlot.f90:520-650, called from ModSave_DoAll :16-59): creates
 * <directory>/AllCells_<step, 8 digits>/ with info.dat and one
 * Block_<global block index, 8 digits>.dat per block, in the reference's text
 * format -- per corner (i fastest, 1..n+1 in each direction) one line of 12
 * ES16.8 values: x, y, z in solar radii, then the 9 variables averaged over the
 * 8 cells around the corner, velocity and B in Cartesian components (Yang
 * blocks mapped as (x, y, z) = (-x0, z0, y0)). The averaging and conversions
 * run on the GPU in batches of blocks; the host writes the text. The state's
 * ghost cells must be current (as after a step or falcon_exchange).
 * 3_6/merge_AllCells.py merges the directory into one Tecplot file. */
int  falcon_save_allcells(falcon_ctx* ctx, const char* directory, int32_t step);
/* Binary restart dump of the device state, which the reference lacks: the
 * raw device arrays (state, the mixed path's 8-bit corrections of u^n, psi
 * with GLM) behind a header with a format version (2: corrections stored for
 * interior cells only), the grid's shape, precision, div-B option, a hash of
 * the block ranges and the step count. falcon_load_restart into a context of
 * the same configuration continues bit for bit as the run that wrote the
 * dump; a file of another configuration or version, or a short file, returns
 * FALCON_ERR_INVALID_ARG and leaves the state unchanged. */
int  falcon_save_restart(falcon_ctx* ctx, const char* path);
int  falcon_load_restart(falcon_ctx* ctx, const char* path);

/* ---- the hot path ------------------------------------------------------- */
int  falcon_exchange(falcon_ctx* ctx);
int  falcon_timestep(falcon_ctx* ctx, double* dt_out);
/* One RK4 step + artificial diffusion. dt_out may be NULL (dt stays on the
 * device). Returns FALCON_ERR_NAN_DETECTED if the wave-speed pass saw a NaN. */
int  falcon_step_rk4(falcon_ctx* ctx, double* dt_out);
/* nsteps back-to-back steps, captured as CUDA graphs after the first call. */
int  falcon_run_steps(falcon_ctx* ctx, int32_t nsteps);
int  falcon_synchronize(falcon_ctx* ctx);
/* ---- block sharding over ranks (one GPU per rank) ------------------------
 * The reference distributes leaf blocks over MPI ranks in contiguous ranges
 * (ModAllocation_Init, 3_6/ModAllocation.f90:25-39) and moves the ghost
 * entries that cross ranks through per-peer packed messages
 * (ModCommunication_SetGC_Sender/Receiver and the exchange,
 * 3_6/ModCommunication.f90:375-634, 725-765), with MIN and SUM allreduces for
 * dt and the CG dot products. Here every rank builds the same tree and ghost
 * map; these entry points give the partition, the per-peer entry lists and,
 * on a sharded context, the pack/unpack of those entries. The transport
 * (NCCL send/recv on GPUs, any message layer) and the MIN of dt are the
 * caller's.
 *
 * falcon_shard_ranges: first[r] .. first[r+1]-1 are rank r's blocks
 * (0-based), r = 0..nranks-1; the first nblocks % nranks ranks get one more.
 * falcon_shard_plan: indices into the falcon_ghost_map order of the entries
 * rank `rank` sends to `peer` (FALCON_SHARD_SEND: source block on rank,
 * target block on peer) or receives from it (FALCON_SHARD_RECV); peer == rank
 * gives the entries within the rank. Both sides list a message's entries in
 * map order, so the sender's pack order is the receiver's. Host-only
 * contexts too.
 *
 * falcon_set_shard (FP64 precision, divb_option 0): this context computes
 * rank `rank`'s blocks. falcon_step_phase then runs over the owned blocks
 * only and fills the ghost entries within the rank; phase 0 accumulates the
 * owned blocks' CFL minimum h/v_wave without forming dt:
 *   per step: phase 0; m = falcon_shard_min_ratio; MIN over ranks;
 *             falcon_shard_set_min_ratio(global m) (dt = min(1e20, CFL m));
 *             for phases 1..5: falcon_step_phase, then for every peer
 *             falcon_shard_pack into the message, and falcon_shard_unpack of
 *             the peer's message.
 * falcon_exchange on a sharded context fills the entries within the rank (the
 * remote ones follow with pack/unpack). Pack buffers hold 8 doubles per entry
 * (falcon_shard_counts gives the entries per peer); a buffer may be host or
 * device memory (a device buffer is written or read in place, ready for a
 * device-side transport). The state's blocks outside the owned range are not
 * updated. */
#define FALCON_SHARD_SEND 0
#define FALCON_SHARD_RECV 1
int  falcon_shard_ranges(const falcon_ctx* ctx, int32_t nranks, int32_t* first);
int  falcon_shard_plan(const falcon_ctx* ctx, int32_t nranks, int32_t rank, int32_t peer, int32_t dir,
                       int64_t* entries, int64_t cap, int64_t* n);
int  falcon_set_shard(falcon_ctx* ctx, int32_t nranks, int32_t rank);
int  falcon_shard_counts(const falcon_ctx* ctx, int32_t peer, int64_t* nsend, int64_t* nrecv);
int  falcon_shard_pack(falcon_ctx* ctx, int32_t peer, double* buf);
int  falcon_shard_unpack(falcon_ctx* ctx, int32_t peer, const double* buf);
int  falcon_shard_min_ratio(falcon_ctx* ctx, double* local_min);
int  falcon_shard_set_min_ratio(falcon_ctx* ctx, double global_min);

/* Poll limit of the step kernels' bounded waits (no counterpart in the
 * reference, whose MPI calls block without a limit). Each stage and diffusion
 * CTA streams its block's planes into shared memory with bulk copies and
 * waits on an mbarrier for each chunk, polling it at most `polls` times
 * (default 4,194,304; each poll may suspend briefly; 0 gives up at once).
 * A wait that runs out ends the CTA cleanly -- uniformly over its threads,
 * after the copies in flight have landed -- and the step returns
 * FALCON_ERR_TIMEOUT (from falcon_step_rk4 with dt_out, falcon_synchronize
 * or falcon_timestep); the state is then undefined until the next
 * falcon_upload_state, falcon_init_synthetic or falcon_load_restart, which
 * clear the flag. polls < 0 restores the default. */
int  falcon_set_wait_limit(falcon_ctx* ctx, int32_t polls);
/* Verification: run one phase of ModAdvance_rk4 eagerly and synchronously.
 * phase 0: wave speed + CFL dt (3_6/ModAdvance.f90:31-48); 1..4: RK stage s
 * with its ghost exchange (:59-97); 5: artificial diffusion + exchange
 * (:101-109). Phases 0,1,2,3,4,5 in order equal one falcon_step_rk4. */
int  falcon_step_phase(falcon_ctx* ctx, int32_t phase);
/* Download the stage buffer (primitive_rk_IV) in the falcon_download_state layout. */
int  falcon_download_stage_state(falcon_ctx* ctx, double* u);

/* ---- measurement -------------------------------------------------------- */
/* Per-kernel CUDA-event timing on the context stream (off by default). */
int  falcon_set_kernel_timing(falcon_ctx* ctx, int32_t on);
/* names: newline-separated kernel names; ms[i], launches[i] per kernel */
int  falcon_kernel_stats(falcon_ctx* ctx, char* names, size_t names_len,
                         double* ms, int64_t* launches, int32_t cap, int32_t* n);
int  falcon_reset_kernel_stats(falcon_ctx* ctx);
/* device-side event timing of the context stream */
int  falcon_timer_start(falcon_ctx* ctx);
int  falcon_timer_stop(falcon_ctx* ctx, double* ms);
/* k-chunk depth (planes per CTA step) chosen for the stage and diffusion
 * kernels. The autotuner runs once per context, before the first step: it
 * times every compiled variant on this grid, on the stage buffer only. */
int  falcon_tuning(falcon_ctx* ctx, int32_t* kpar_stage, int32_t* kpar_diffusion);
/* fix the k-chunk depths instead (no autotuning): one of the compiled
 * variants, FP32 16^3 blocks 1, 2 or 4 (for the diffusion pass: 1 = one
 * thread per cell column, 2 or 4 = two), FP32 8^3 blocks 2, 4 or 8, FP64 1
 * (16^3) or 2, 4 (8^3); anything else is FALCON_ERR_INVALID_ARG. Every
 * variant computes the same values bit for bit. */
int  falcon_set_tuning(falcon_ctx* ctx, int32_t kpar_stage, int32_t kpar_diffusion);
/* How falcon_step_rk4 runs a step. FALCON_STEP_GRAPH (default): one captured
 * CUDA graph of 11 launches (dt, 4 stages and their exchanges, diffusion, the
 * final exchange). FALCON_STEP_PERSISTENT: one persistent cooperative launch
 * that runs the same kernel bodies over all blocks with a bounded grid
 * barrier between the phases (a barrier wait that runs out makes the step
 * return FALCON_ERR_TIMEOUT); the same values bit for bit. The persistent
 * step covers the mixed path with 16^3 blocks and divb_option 0; other
 * contexts return FALCON_ERR_INVALID_ARG. */
#define FALCON_STEP_GRAPH      0
#define FALCON_STEP_PERSISTENT 1
int  falcon_set_step_mode(falcon_ctx* ctx, int32_t mode);
/* device ghost-fill lists: counts[0] exact copies, [1] 1-D blends, [2] trilinear/rotated */
int  falcon_ghost_list_sizes(const falcon_ctx* ctx, int64_t* counts);
/* the exchanges between RK stages (face ghosts only; every stencil of a step
 * is axis-aligned, the exchange that ends the step fills edges and corners):
 * out[0..2] list sizes as above, out[3] block faces whose ghosts the stage
 * kernel writes directly (mixed mode), out[4] ghost cells on those faces */
int  falcon_exchange_stats(const falcon_ctx* ctx, int64_t* out5);
/* bytes of device memory held by the context */
int  falcon_device_bytes(const falcon_ctx* ctx, int64_t* bytes);

/* ======================================================================
 * Implicit solvers: multigrid-preconditioned flexible CG on the Yin-Yang
 * grid (replaces ModPFSS_setup/ModPFSS_solve, 3_5/ModPFSS.f90:21-150, and
 * ModLinearSolver_Multigrid_CG, 3_5/ModLinearSolver.f90:313-427; the
 * conduction operator fills the empty ModHeatConduction, 3_6/ModHeatConduction.f90).
 * ====================================================================== */
#define FALCON_MAX_PROBLEMS 256
#define FALCON_SOLVER_PFSS        0   /* Laplace solve, source surface at r_range[1] */
#define FALCON_SOLVER_CONDUCTION  1   /* backward-Euler anisotropic heat conduction */
#define FALCON_PRECOND_NONE 0
#define FALCON_PRECOND_MG   1         /* one FP32 V-cycle (red-black Gauss-Seidel) */
/* one V-cycle whose coarsest-level smoothing is replaced by the learned
 * coarse correction (falcon_solver_attach_lcc) followed by a few sweeps;
 * falls back to FALCON_PRECOND_MG for the rest of a solve that stagnates */
#define FALCON_PRECOND_MG_LCC 2

typedef struct falcon_solver_spec {
    int32_t  kind;                     /* FALCON_SOLVER_* */
    int32_t  nproblems;                /* independent problems solved in one batch */
    int32_t  block;                    /* cells per block edge (even) */
    int32_t  nlevels;                  /* multigrid levels (capped by the block size) */
    int32_t  device;                   /* CUDA device; < 0 builds the host side only */
    int32_t  pad_;
    uint64_t seed;                     /* problem q uses seed + q */
    double   r_range_rsun[2];          /* PFSS: [1.0, 2.5]; conduction: [0.7, 1.0] */
    double   dt_factor;                /* conduction: dt in units of the explicit limit */
    /* PFSS: nr[q], nt[q] (ntheta; nphi = 2 ntheta), mapped to per-panel
     * (nr, nt/2, 3 nt/2) rounded up to whole blocks. Conduction: per-panel
     * cells nr[0] x nt[0] x np[0] (np = 3 nt). */
    int32_t  nr[FALCON_MAX_PROBLEMS];
    int32_t  nt[FALCON_MAX_PROBLEMS];
    int32_t  np[FALCON_MAX_PROBLEMS];
} falcon_solver_spec;

/* A solve is an FP64 iterative refinement: r = b - A x and its norms in FP64,
 * an inner flexible-CG solve (float-float vectors, FP32 V-cycle) of the
 * correction equation A d = r, x += d in FP64; a problem is converged only
 * when its FP64 ||b - A x|| / ||b|| <= tol. Every problem of the batch is
 * advanced by the same launches, and each inner solve is one CUDA-graph
 * launch: a first iteration and a conditional WHILE node whose body is one
 * iteration (V-cycle included), looping on the device until every problem
 * reaches its inner tolerance, the residual stalls or the iteration budget
 * runs out (bounded). falcon_solver_solve returns FALCON_OK only when every
 * problem converged, FALCON_ERR_NOT_CONVERGED otherwise (the report is
 * filled either way). */
typedef struct falcon_solve_report {
    int32_t iterations;                /* inner iterations, all refinement passes */
    int32_t converged;                 /* 1: every problem's FP64 relative residual <= tol */
    int32_t vcycles;
    int32_t refinements;               /* refinement passes after the first */
    double  rel_residual;              /* max over problems of the FP64 ||b-Ax||/||b|| at exit */
    double  ms;                        /* device time of the solve */
    int32_t fallbacks;                 /* FALCON_PRECOND_MG_LCC: switches to plain MG */
    int32_t pad_;
    /* > 0 when a problem stopped above tol because FP64 cannot take it lower:
     * its residual is at the attainable accuracy of b - A x, 4 x 8 eps64
     * (|b| + |A||x|) / ||b||, or a refinement pass no longer halved it (the
     * largest such residual; converged is then 0) */
    double  floor_residual;
} falcon_solve_report;

typedef struct falcon_solver falcon_solver;
typedef struct falcon_lcc falcon_lcc;   /* learned coarse correction (below) */

int  falcon_solver_create(falcon_solver** out, const falcon_solver_spec* spec);
void falcon_solver_destroy(falcon_solver* sv);
int  falcon_solver_last_error(const falcon_solver* sv, char* buf, size_t len);
/* info: nblocks, nproblems, nlevels, m_i, m_j, m_k (level-0 cells per block) */
int  falcon_solver_info(const falcon_solver* sv, int32_t* info);
/* first[q] = first global block of problem q, q = 0..nproblems */
int  falcon_solver_problem_blocks(const falcon_solver* sv, int32_t* first);
/* level-0 right-hand side [block][k][j][i] */
int  falcon_solver_rhs(const falcon_solver* sv, double* b);
/* face-coefficient operator of a level (3_5/ModBlock.f90:39-44 layout, C order
 * [block][k][j][i]; Ai has m_i+1 faces along i, Aj m_j+1 along j, Ak m_k+1 along k) */
int  falcon_solver_operator(const falcon_solver* sv, int32_t level, double* Aii, double* Ai, double* Aj, double* Ak);
int  falcon_solver_halo_count(const falcon_solver* sv, int32_t level, int64_t* n);
/* idx[n][8] = tb,ti,tj,tk,sb,i0,j0,k0 ; wx[n][6] = weights (3), source-frame centre (3) */
int  falcon_solver_halo_map(const falcon_solver* sv, int32_t level, int32_t* idx, double* wx);
/* y = A x on the GPU (level 0, halo filled on the device) */
int  falcon_solver_apply(falcon_solver* sv, const double* x, double* y);
int  falcon_solver_solve(falcon_solver* sv, double tol, int32_t max_iter, int32_t precond, falcon_solve_report* rep);
int  falcon_solver_solution(falcon_solver* sv, double* x);
/* conduction time step dt (dt_factor x the explicit stability limit) */
int  falcon_solver_timestep(const falcon_solver* sv, double* dt);
/* red-black Gauss-Seidel sweeps of the V-cycle: before and after the coarse
 * correction on every level but the coarsest, and on the coarsest level
 * (defaults 1, 1, 32 for PFSS; 2, 2, 4 for conduction, whose implicit step
 * makes the coarse problem well conditioned: fewer coarse sweeps leave its
 * iteration count unchanged) */
int  falcon_solver_set_smoothing(falcon_solver* sv, int32_t nu_pre, int32_t nu_post, int32_t nu_coarse);
/* FP64 true relative residual ||b - A x|| / ||b|| of every problem for the
 * current solution (rel[nproblems]) */
int  falcon_solver_problem_residuals(falcon_solver* sv, double* rel);
/* replace the level-0 right-hand side [block][k][j][i] */
int  falcon_solver_set_rhs(falcon_solver* sv, const double* b);
/* ---- the driver's own data (a solver created from a spec is then only the
 * grid: its seeded synthetic operator or magnetogram is replaced) ---- */
/* Replace the level-0 operator with the driver's face coefficients, the
 * layout of falcon_solver_operator (Aii[b][k][j][i], Ai[b][k][j][m_i+1],
 * Aj[b][k][m_j+1][i], Ak[b][m_k+1][j][i]; 3_5/ModBlock.f90:39-44), e.g. the
 * backward-Euler conduction operator a driver assembled from its own T and B
 * (ModHeatConduction, 3_6/ModHeatConduction.f90, is empty in the reference).
 * The coarse levels are rebuilt (Galerkin) and every device copy refreshed.
 * Rejected, operator unchanged, unless every coefficient is finite and every
 * Aii positive. */
int  falcon_solver_set_operator(falcon_solver* sv, const double* Aii, const double* Ai, const double* Aj,
                                const double* Ak);
/* PFSS: the lower-boundary radial field Br at the bottom faces of the level-0
 * bottom blocks, br[b][k][j] (m_k x m_j per block; entries of other blocks
 * are ignored) -- the driver's magnetogram in place of the synthetic one
 * (ModPFSS_setup's Block%magnetogram_LL, 3_5/ModPFSS.f90:21-100, filled by
 * ModMagnetogram, 3_5/ModMagnetogram.f90:13-80). The right-hand side becomes
 * b(1,:,:) = Br * S_i(1,:,:) (3_5/ModPFSS.f90:45-48). Rejected, unchanged,
 * if any value is not finite or the solver is not a PFSS solver. */
int  falcon_solver_set_magnetogram(falcon_solver* sv, const double* br);
/* the current PFSS magnetogram in the same layout (0 off the bottom blocks) */
int  falcon_solver_magnetogram(const falcon_solver* sv, double* br);
/* Tile shape of the solver's cell kernels: each CTA takes a chunk of a
 * block's cells (never two blocks, so its reductions go to one problem).
 * Chosen by the solver's autotuner at its first solve -- every candidate
 * (cells per CTA 512..4096 that are multiples of the row length, threads per
 * CTA 128, 256 or 512) timed on one eager FCG iteration of this grid.
 * tile[0] cells per CTA, tile[1] threads per CTA, tile[2] 1 once tuned or
 * set; ms_per_iteration (may be NULL) the timed iteration of the choice.
 * falcon_solver_set_tile fixes the shape instead (no autotuning). */
int  falcon_solver_tuning(const falcon_solver* sv, int32_t* tile, double* ms_per_iteration);
int  falcon_solver_set_tile(falcon_solver* sv, int32_t cells_per_cta, int32_t threads_per_cta);
/* Verification: one kernel of the V-cycle on host arrays at `level`, eagerly
 * and synchronously (as falcon_step_phase is for the step). Arrays are FP32,
 * interior cells [block][k][j][i] of their level.
 *   RESTRICT:   in0 = fine residual (level) -> out = coarse right-hand side
 *               (level+1), the sum of each cell's 8 children in the order of
 *               ModMath_rebin_3D_factor2 (3_6/ModMath.f90:353-368) without its
 *               /8 (the operators are volume-integrated: R = P^T)
 *   PROLONG_ADD: in0 = coarse correction (level+1), in1 = fine correction
 *               (level) -> out = in1 + injection of in0
 *               (ModMath_prolongate_3D_factor2, 3_6/ModMath.f90:370-384)
 *   SMOOTH_RED / SMOOTH_BLACK: in0 = r, in1 = z -> out = z after one
 *               red-black Gauss-Seidel half sweep of that colour (cells with
 *               i+j+k even / odd) with the halo filled from z first; each
 *               updated cell takes the Jacobi formula of
 *               ModMultigrid_Jacobi_Mz_r (3_5/ModMultigrid.f90:316-324)
 *   RESIDUAL:   in0 = r, in1 = z -> out = r - A z (halo filled from z) */
#define FALCON_VCYCLE_RESTRICT     0
#define FALCON_VCYCLE_PROLONG_ADD  1
#define FALCON_VCYCLE_SMOOTH_RED   2
#define FALCON_VCYCLE_SMOOTH_BLACK 3
#define FALCON_VCYCLE_RESIDUAL     4
int  falcon_solver_vcycle_op(falcon_solver* sv, int32_t op, int32_t level, const float* in0, const float* in1,
                             float* out);
/* level-0 block geometry, for a driver that evaluates its own fields on the
 * grid: ranges[b][3][2] (r in cm, theta, phi in the block's panel frame) and
 * flags[b] (bit0 Yin, bit1 top, bit2 bottom), blocks of all problems in order */
int  falcon_solver_block_ranges(const falcon_solver* sv, double* ranges);
int  falcon_solver_block_flags(const falcon_solver* sv, int32_t* flags);
/* PFSS: the point charges of problem `problem`'s synthetic magnetogram,
 * xyzq[n][4] = x, y, z (cm, Yin frame) and signed charge, in pole pairs
 * (+q, -q) of the tilted bipoles; *n receives the count (xyzq may be NULL to
 * query it). The synthetic Br at a bottom face centre (r, theta, phi), Yin
 * frame, is the ModMagnetogram sum (3_5/ModMagnetogram.f90:43-74) over these
 * charges plus a 1 G axial dipole, cos(theta). */
int  falcon_solver_magnetogram_sources(const falcon_solver* sv, int32_t problem, double* xyzq, int32_t cap,
                                       int32_t* n);
/* initial guess x0 of the next solves, level 0 [block][k][j][i] (PFSS
 * default 0; conduction default the current temperature) */
int  falcon_solver_set_guess(falcon_solver* sv, const double* x0);
/* Learned coarse correction (single-problem solvers of whole uniform blocks):
 * the coarsest level gathered into one dense grid per Yin-Yang panel,
 * shape4 = {2, D, H, W} (D radial, H theta, W phi cells; multiples of 8). */
int  falcon_solver_coarse_shape(falcon_solver* sv, int32_t* shape4);
/* use `net` in FALCON_PRECOND_MG_LCC solves, followed by `sweeps` red-black
 * Gauss-Seidel sweeps at the coarsest level (the network stays owned by the
 * caller and must outlive its use) */
int  falcon_solver_attach_lcc(falcon_solver* sv, falcon_lcc* net, int32_t sweeps);
/* Training pairs from a real solve: runs an MG-preconditioned FCG solve and
 * records the coarsest-level residual r_c of each V-cycle (up to
 * max_records); for each, solves A_c e_c = r_c to 1e-6 (Jacobi-PCG, FP64)
 * and writes the network input x[2 r][D][H][W][8] (r_c/diag scaled by its RMS
 * s, then the six face couplings / diag and the diagonal surplus / diag) and
 * the target t[2 r][D][H][W] = e_c / s. nrecords receives r. */
int  falcon_solver_record(falcon_solver* sv, double tol, int32_t max_iter, int32_t max_records, float* x, float* t,
                          int32_t* nrecords);

/* ---- learned coarse correction (no counterpart in the reference) --------
 * A 4-level 3D convolutional U-Net that predicts the coarsest-level error of
 * the conduction V-cycle from the coarsest-level residual and operator, used
 * as a preconditioner stage inside the flexible CG (ModLinearSolver_
 * Multigrid_CG, 3_5/ModLinearSolver.f90:313-427, is the method it extends).
 * Input x[n][D][H][W][FALCON_LCC_CIN] (FP32, channels last; D, H, W multiples
 * of 8), output y[n][D][H][W]. Layers (3x3x3 convolutions, zero padding,
 * ReLU on all but the last): 8->16, 16->16 | pool | 16->32, 32->32 | pool |
 * 32->64 | pool | 64->64 | up + skip | 64->32 | up + skip | 32->16 | up + skip
 * | 16->16, 16->1. Parameters: per layer W[co][ci][27] (tap = (kd*3+kh)*3+kw)
 * then b[co], concatenated. BF16 weights and activations on tensor cores with
 * FP32 accumulation; FP32 master weights trained with Adam on a mean-square
 * loss. */
#define FALCON_LCC_CIN 8
int  falcon_lcc_create(falcon_lcc** out, int32_t device, uint64_t seed);
void falcon_lcc_destroy(falcon_lcc* net);
int  falcon_lcc_last_error(const falcon_lcc* net, char* buf, size_t len);
int  falcon_lcc_num_params(const falcon_lcc* net, int64_t* n);
int  falcon_lcc_get_params(falcon_lcc* net, float* params);
int  falcon_lcc_set_params(falcon_lcc* net, const float* params);  /* also resets Adam */
int  falcon_lcc_forward(falcon_lcc* net, const float* x, int32_t n, int32_t D, int32_t H, int32_t W, float* y);
/* mean-square loss against t[n][D][H][W] and its gradient for every parameter */
int  falcon_lcc_loss_grad(falcon_lcc* net, const float* x, const float* t, int32_t n, int32_t D, int32_t H, int32_t W,
                          double* loss, float* grad);
/* epochs of Adam over nsamples (x, t) pairs in shuffled minibatches of `batch`;
 * epoch_loss[epochs] receives the mean training loss of each epoch */
int  falcon_lcc_train(falcon_lcc* net, const float* x, const float* t, int32_t nsamples, int32_t D, int32_t H,
                      int32_t W, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* epoch_loss);
/* Tensor-core path of the convolutions (forward, backward data and weight
 * gradients): FALCON_LCC_TCGEN05, the default (5th-generation tensor cores:
 * tcgen05.mma with the FP32 accumulator in tensor memory, operands staged in
 * shared memory, weight and activation tiles brought in by TMA), or
 * FALCON_LCC_MMA_SYNC (warp-level mma.sync). Same BF16 operands and FP32
 * accumulation; sums may differ in the last bits of their order. A tcgen05
 * kernel's bounded wait that runs out makes the call return
 * FALCON_ERR_TIMEOUT. */
#define FALCON_LCC_MMA_SYNC 0
#define FALCON_LCC_TCGEN05  1
int  falcon_lcc_set_tensor_path(falcon_lcc* net, int32_t path);
/* Poll limit of the tcgen05 kernels' mbarrier waits (default 4,194,304;
 * polls < 0 restores it). A wait that runs out ends the tile: its copies and
 * MMAs in flight are drained with the default bound before its tensor memory
 * is freed, its results are discarded, and the call returns
 * FALCON_ERR_TIMEOUT. */
int  falcon_lcc_set_wait_limit(falcon_lcc* net, int32_t polls);

#ifdef __cplusplus
}
#endif
#endif /* FALCON_GB300_H */
