// nb_internal.h -- handle state shared by the host orchestration and the kernel files.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "moil_nb.h"
#include "nb_common.cuh"

// FFT plan for one length: radices (4, 2, 3, 5 in that order), twiddles exp(-2 pi i k / n)
// at tw0, and per Stockham stage s: the span Ns, the butterfly count nb = n/R, the magic
// multiplier for dividing by nb, and nb (twiddle step, destination index) entries at tab0+off[s]
struct FftPlanDev {
    int n, nst, tw0, tab0;
    int rad[8];
    int ns[8];
    int nb[8];
    int off[8];
    unsigned magic[8];
};

struct RepHost {
    moil_nb_params p;
    int npt;
    double alpha;
    std::vector<double> q, e6, e12;
    std::vector<int> exc1, exc2, spec1, spec2, poipt, montype;
    std::vector<double> p14;
    int nwat;
    int nuniq_oth;
};

struct NbCtx {
    int device = 0;
    int nsm = 152;                // multiprocessors: grids of the rebuild-gated kernels stay one wave
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // PME branch of an evaluation, concurrent with the pair kernels
    cudaStream_t sbody = nullptr;     // captures the list rebuild into the conditional node's body
    cudaStream_t sstep = nullptr;     // captures an MD step into its gate node's body
    int capturing = 0;                // the evaluation is being captured into the handle's graph
    cudaStream_t pstream = nullptr, pstream2 = nullptr;   // replica groups: prioritised by group index
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int precision = MOIL_NB_MIXED;
    int inited = 0;
    std::string err;

    // replicas
    int nrep = 0;
    std::vector<RepHost> rh;
    std::vector<RepDev> rd;
    RepDev *d_reps = nullptr;
    int64_t natom = 0, nW = 0, nA = 0, nsite = 0, nunit = 0;
    float skin = 1.0f, rwat = 1.1f;
    int list_period = 0;
    int water_excl_fast = 0;      // every water's exclusions are exactly O-H1, O-H2, H1-H2

    // static per caller atom
    double *d_q = nullptr;        // charges
    float2 *d_lj_f = nullptr;     // (epsgm12, epsgm6) per caller atom, FP32 copy
    double2 *d_lj_d = nullptr;    // FP64 copy
    unsigned *d_aflags = nullptr; // SF_* per caller atom
    int *d_atom_rep = nullptr;

    // units
    int *d_unit_atom = nullptr;   // first caller atom of each unit (waters first, then others)
    int *d_unit_rep = nullptr;
    int ncell = 0;                // total cells over replicas
    int *d_unit_key = nullptr, *d_unit_slot = nullptr;
    int *d_bin_count = nullptr, *d_bin_start = nullptr;   // 2*ncell bins (+1)
    int *d_sorted_unit = nullptr;

    // site arrays
    int *d_site_orig = nullptr, *d_site_of = nullptr, *d_site_rep = nullptr;
    unsigned *d_site_flags = nullptr;
    void *d_pos = nullptr;        // float4 / double4 (x, y, z, q_eff)
    float4 *d_posb = nullptr;     // positions at the last list build
    void *d_woff = nullptr;       // float4 / double4 per water, 3 in a row: O position (and charge),
                                  // then the two H offsets from O (FP64-computed)
    void *d_site_lj = nullptr;    // float2 / double2
    void *d_site_q = nullptr;     // float / double (PME charge)

    // pair lists (CSR)
    int2 *d_wl1_cnt = nullptr;    // W1 row counts (in-cutoff from the front, skin-only from the back)
    int *d_wl1 = nullptr;         // W1 rows of cap_row1 entries: sorted water index of j (int32), or
                                  // with row16 its offset from the replica's first water (uint16)
    int row16 = 0;                // every replica has fewer than 65,536 waters
    int cap_row1 = 0;
    int *d_wl2_off = nullptr, *d_wl2 = nullptr;
    int *d_xl_off = nullptr, *d_xl = nullptr;
    int64_t cap_wl2 = 0, cap_xl = 0;
    int *d_count_tmp = nullptr;   // scratch counts
    long long *d_scan_tmp = nullptr;   // tile sums of the three-phase scan
    std::vector<int2> wtiles;     // (replica, first sorted water) of each tiled water-list block
    int2 *d_wtiles = nullptr;
    // half water rows (FP32 path with 16-bit rows: k_whalf builds them, k_water_h reads them)
    int whalf = 0;                // the half-list water kernel is in use
    int want_whalf = 0;           // MOIL_NB_WATER_*: 0 automatic, 1 full lists, 2 half lists
    int hb = 256;                 // waters per half-list block (128, 256 or 512)
    int want_tiled = 0;           // MOIL_NB_TILED_*
    std::vector<int2> hblocks;    // (replica, first sorted water) of each half-list block
    int2 *d_hblocks = nullptr;
    unsigned *d_hrow = nullptr;   // caph entries per lane, entry k of lane t at k * hb + t per block
    int2 *d_hcnt = nullptr;       // per water: owned in-cutoff entries, owned entries
    int *d_jset = nullptr;        // per block: jcap sorted water indices (the block's partners)
    int *d_jn = nullptr;          // per block: j-set size
    int caph = 0, jcap = 0;

    // exclusion / 1-4 lists per caller atom (both directions)
    int *d_ex_off = nullptr, *d_ex_j = nullptr;
    int *d_p14_off = nullptr, *d_p14_j = nullptr;
    double *d_p14_par = nullptr;

    // outputs
    long long *d_grad_site = nullptr;  // nsite*3 fixed point
    double *d_e_unit = nullptr;        // nunit*4
    double *d_grad_ex = nullptr;       // natom*3
    double *d_e_ex = nullptr;          // natom*3

    // PME
    std::vector<FftPlanDev> plans;
    FftPlanDev *d_plans = nullptr;
    std::vector<int> rep_plan;         // 3 plan indices per replica
    int *d_rep_plan = nullptr;
    void *d_tw = nullptr;              // float2 / double2 twiddles
    int2 *d_tab = nullptr;             // Stockham stage tables (twiddle step, destination index)
    std::vector<double> bsp_h;
    void *d_bsp = nullptr;             // float / double moduli
    float *d_etab = nullptr;           // FP32 path: exp(-pi^2 m^2 / (alpha L)^2) / B per dimension (bsp layout)
    int nzbin = 0;
    int *d_zcount = nullptr, *d_zstart = nullptr, *d_zslot = nullptr, *d_zatoms = nullptr;
    void *d_fr = nullptr;              // float4 / double4 per site (fr1, fr2, fr3, q*fc)
    void *d_grid = nullptr;            // half-complex grids, float2 / double2
    int64_t grid_elems = 0;
    void *d_part = nullptr;            // per site 4 slots x 3 (float / double)
    std::vector<PlaneWork> planes;
    PlaneWork *d_planes = nullptr;
    std::vector<ColWork> cols;
    ColWork *d_cols = nullptr;
    std::vector<int> col_begin;        // per replica, nrep+1
    int *d_col_begin = nullptr;
    double *d_e_col = nullptr;         // energy partial per column work item
    size_t smem_plane_fwd = 0, smem_plane_inv = 0, smem_zconv = 0;
    int max_n1 = 0, max_n2 = 0, max_n3 = 0;

    // energies
    std::vector<EChunk> echunks;       // fixed partition of the energy partials (k_energy_part)
    EChunk *d_echunks = nullptr;
    int *d_echunk_begin = nullptr;     // first chunk of each replica, then the count
    double *d_epart = nullptr;         // NB_EU slot sums per chunk
    double *d_e_rep = nullptr;         // nrep * 16
    double *h_e_rep = nullptr;         // pinned mirror

    // caller buffers used by host-pointer evaluations
    double *d_coor = nullptr, *d_dpot = nullptr;
    double *d_adj = nullptr;           // parameter derivatives, 3 x natom (allocated on first use)
    double *d_adj_phi = nullptr;       // plain path: PME potential share of 4 planes per site (first use)
    double *d_md_dpot = nullptr;       // gradient of the MD steps (moil_nb_md_step, first use)
    // device-side MD step loop (moil_nb_md_step): one graph per context holds a whole step
    // (evaluation, then leapfrog + SETTLE); d_mdctl = {evaluations since the last rebuild,
    // rebuild requested, sticky error bits}, read back once per call
    cudaGraphExec_t gexec_md = nullptr;
    const void *gmd_key[3] = {nullptr, nullptr, nullptr};
    double gmd_dt = 0.0, gmd_doh = 0.0, gmd_dhh = 0.0;
    int gmd_gen = -1;
    double *gmd_dpot = nullptr;
    int *d_mdctl = nullptr;
    double *d_md_save = nullptr;       // the call's starting coordinates and velocities (the
                                       // per-step path redoes the call from them after an error)

    // pressure analysis (moil_nb_set_molecules / moil_nb_pressure, nb_press.cu)
    int nmol = 0;
    int *d_mol_off = nullptr, *d_mol_atom = nullptr;   // molecules as CSR over caller atoms
    double *d_mass = nullptr;          // per caller atom
    double *d_xrel = nullptr;          // position relative to the molecule's centre of mass, 3 per atom
    void *d_xsite = nullptr;           // the same in site order, float4 / double4 (pair kernels)
    double *d_press_unit = nullptr;    // 6 per unit: LJ and real-space Coulomb terms
    double *d_press_site = nullptr;    // 3 per site: PME force x xrel
    double *d_press_col = nullptr;     // 3 per PME column work item: reciprocal virial
    void *d_press_grid = nullptr;      // second half-complex grid for the reciprocal virial (float2 / double2)
    double *d_press_out = nullptr;     // 12 per replica

    // device status: [0] rebuild flag, [1] error bits, [2..4] W1 / W2 / X entry totals,
    // [5] largest half-list j-set, [6] longest W1 row, [7] longest half row; all reset at the
    // start of every evaluation
    int *d_status = nullptr;
    int *h_status = nullptr;           // pinned: [0..7] mirror, [8..15] initial words of an evaluation,
                                       // [16] the rebuild flag read back in stage-timing mode,
                                       // [17..19] / [20..22] MD step control written / read back
    int need_rebuild = 1;
    int evals_since_build = 0;
    int64_t last_list_entries = 0, last_water_pairs = 0, last_atom_pairs = 0, last_site_pairs = 0;

    // instrumentation
    int timing = 0;
    // stage events: 0 start, 12 prepared, 13 rebuild decided, 1 lists, 2..5 pair kernels,
    // 6..9 PME, 10 end; 11 orders the replica groups after their shared input copies
#define NB_NEV 14
    cudaEvent_t ev[NB_NEV];
    moil_nb_timing last_timing{};
    int launches = 0;

    // CUDA graph of one evaluation, valid for the caller pointers and list buffers it captured
    int use_graph = 1;
    int virial = 0;                    // water-water LJ virial in the FP32 water kernel

    // replica groups (nb_host.cu): a batch evaluated as concurrent contiguous replica ranges,
    // each a complete context; this context then holds no device buffers of its own
    std::vector<NbCtx *> grp;
    std::vector<int> grp_rep0;         // first replica of each group, then nrep
    std::vector<int64_t> grp_atom0;    // first caller atom of each group, then natom
    int want_groups = 0;               // 0: automatic, 1: none, P: P groups (next init)
    std::string tune_cache;            // autotuner cache file read by moil_nb_init_batch ("" none)
    int tuning = 0;                    // moil_nb_autotune is re-initialising the handle
    int tune_mode = 0;                 // MOIL_NB_TUNE_DEVICE / MOIL_NB_TUNE_HOST
    cudaGraphExec_t gexec = nullptr;
    const double *g_coor = nullptr;
    double *g_dpot = nullptr;
    int g_gen = -1, list_gen = 0, graph_launches = 0;
    // an asynchronous evaluation queued by moil_nb_eval_device_async and not yet waited for
    int pending = 0, pend_rc = 0;
    const double *pend_coor = nullptr;
    double *pend_dpot = nullptr;
    int on_prio = 0, g_prio = 0;       // running on the prioritised group streams (now / when captured)
};

// the public handle is the context itself
struct moil_nb_ctx : NbCtx {};

// a cached shape for this batch (nb_tune.cu), applied to h's requested shapes; 1 if found
int nb_tune_cached_shape(moil_nb_ctx *h, int nrep, const moil_replica *reps);

// list capacity as the int the kernels compare CSR offsets against
inline int cap_int(int64_t cap) { return cap > 0x7fffffff ? 0x7fffffff : (int)cap; }

// ---- launchers implemented in the kernel files -------------------------------------
// lists (nb_lists.cu)
void nb_launch_build_lists(NbCtx *c, const double *d_coor);
// one thread sets the conditional node of a captured evaluation to the device rebuild flag
void nb_launch_rebuild_cond(NbCtx *c, cudaGraphConditionalHandle h);
void nb_launch_prepare(NbCtx *c, const double *d_coor, int check);
void nb_exclusive_scan(NbCtx *c, const int *d_in, int *d_out, int n, int *d_total);
// real space + corrections (nb_realspace.cu)
void nb_launch_realspace(NbCtx *c);
// half-list water kernel: dynamic shared memory for c->jcap; MOIL_NB_OK if it fits the device
int nb_half_configure(NbCtx *c);
// the half-list kernel still fits its two (256-water) or four (128) resident blocks per SM
bool nb_half_two_blocks(NbCtx *c);
// shared-memory carveouts of the full-list water kernels
int nb_realspace_configure(NbCtx *c);
void nb_launch_excl14(NbCtx *c, const double *d_coor);
// PME (nb_pme.cu)
void nb_launch_pme(NbCtx *c);
int nb_pme_configure(NbCtx *c);
// |DFT|^2 of the order-4 B-spline (pot/ewald_receip.f:413-481), n values
void nb_bsp_moduli(int n, double *mod);
// int32 PME plane scale 2^nb_spread_exp(max |q| fc), its inverse and the FP32 spread factor
void nb_spread_scale(double qfc_max, RepDev *R);
// FP32-path constants of the influence function from pme_fac, pivol and invLd
void nb_pme_fp32_consts(RepDev *R);
// FP32-path influence-function table of one replica (n1 + n2 + n3 entries, bsp layout) from its
// FP64 B-spline moduli
void nb_pme_etab(const RepDev &R, const double *bsp, float *out);
// finalize (nb_realspace.cu)
void nb_launch_finalize(NbCtx *c, double *d_dpot);
// MD step loop (nb_md.cu / nb_host.cu): the step-control kernels around an evaluation, the
// integrator of one context, and the graph replay of nsteps whole steps (no host wait)
void nb_launch_md_begin(NbCtx *c, cudaStream_t s);
void nb_launch_md_gate(NbCtx *c, cudaStream_t s, cudaGraphConditionalHandle h);
void nb_launch_md_end(NbCtx *c, cudaStream_t s);
int nb_launch_integrate(NbCtx *c, cudaStream_t s, double *coor, double *vel, const double *mass, const double *dpot,
                        double dt, double doh, double dhh);
int nb_md_loop(NbCtx *c, double *coor, double *vel, const double *mass, double *dpot, double dt, double doh,
               double dhh, int nsteps);
// per-replica energies and pair count of the last completed evaluation (e may be NULL)
void read_energies_of(NbCtx *c, moil_energies *e);
// parameter derivatives after an evaluation of c->d_coor (nb_adjoint.cu), mixed path
int nb_adjoint(NbCtx *c, double *d_dq, double *d_de, double *d_ds);
// pressure analysis terms after an evaluation of d_coor (nb_press.cu): 12 per replica
int nb_pressure(NbCtx *c, const double *d_coor, double *d_out);

#define NB_CUDA_OK(c, call)                                                         \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            (c)->err = std::string(#call) + ": " + cudaGetErrorString(e_);          \
            return MOIL_NB_ERR_CUDA;                                                \
        }                                                                           \
    } while (0)
