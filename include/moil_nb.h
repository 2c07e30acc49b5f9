/*
 * moil_nb.h -- C ABI of the GB300 nonbonded energy/force library.
 *
 * Drop-in for the nonbonded Ewald block of MOIL's eforce() (pot/eforce.f:122-204):
 * real-space LJ + erfc-Coulomb over the pair lists (pot/cdie_ewald.f,
 * pot/watwat_ewald.f, symm/symcdie_ewald.f, symm/symwat_ewald.f), the exclusion
 * erf corrections (pot/cdie_ewald.f:117-199), the 1-4 terms (pot/ener14.f), the
 * PME reciprocal sum (pot/ewald_receip.f) and the self energy
 * (symm/ewald_init.f:131-150), plus the list rebuild that MOIL does in
 * squeeze()/nbondm()/syminit() (symm/squeeze.f, pot/nbondm.f, symm/syminit.f).
 *
 * Conventions follow MOIL's COMMON blocks:
 *   - coordinates coor(3,npt) and gradients dpot(3,npt) are interleaved x,y,z
 *     per atom (Fortran column-major), Å and kcal/mol/Å; dpot = dE/dx (-force);
 *   - atom numbers inside index arrays (exc2, spec1/2, poipt) are 1-based as
 *     MOIL stores them;
 *   - energies are kcal/mol and fill the same names as /ENERGY/ and /EWALD3/.
 *
 * Every call returns an int status (MOIL_NB_OK == 0) and never aborts: MOIL's
 * alert(...,1) is the caller's decision (pot/nbond.f:164-173).  A handle is
 * not thread safe; use one handle per host thread.
 */
#ifndef MOIL_NB_H
#define MOIL_NB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    MOIL_NB_OK = 0,
    MOIL_NB_ERR_ARG = 1,          /* bad pointer / size / handle */
    MOIL_NB_ERR_CUDA = 2,         /* CUDA runtime error (message via moil_nb_last_error) */
    MOIL_NB_ERR_NONNEUTRAL = 3,   /* |sum q| > 1e-7: symm/ewald_init.f:62-72 */
    MOIL_NB_ERR_GRID = 4,         /* PME grid not 2/3/5-smooth, > 128 per side, or order != 4 */
    MOIL_NB_ERR_BOX = 5,          /* cutoff + water extent does not fit half the box */
    MOIL_NB_ERR_OVERFLOW = 6,     /* device list capacity exceeded (retry grows it) */
    MOIL_NB_ERR_NAN = 7,          /* non-finite coordinate or result */
    MOIL_NB_ERR_TOPOLOGY = 8,     /* water monomer not O,H,H with full intramolecular exclusions */
    MOIL_NB_ERR_TIMEOUT = 9,      /* a bounded device wait expired */
    MOIL_NB_ERR_NOMEM = 10,
    MOIL_NB_ERR_STATE = 11        /* call order (e.g. eval before init) */
};

/* precision of the device path */
enum {
    MOIL_NB_MIXED = 0,            /* FP32 pair/spline/FFT math, int64 fixed-point force accumulation,
                                     FP64 energies, exclusion/1-4 corrections and self energy */
    MOIL_NB_FP64 = 1              /* plain FP64 throughout, one system per launch (baseline path) */
};

/* monomer kinds (moname in MOIL) */
enum {
    MOIL_MON_OTHER = 0,           /* solute residue: never squeezed */
    MOIL_MON_WATER = 1,           /* 'TIP3' / 'SPC*': O,H,H; O-O group cutoff (pot/nbondm.f:189-199) */
    MOIL_MON_ION = 2              /* squeezed single-molecule monomer (symm/squeeze.f:82-86) */
};

/* Run parameters: the keywords pot/energy.f:188-253 reads, plus device knobs. */
typedef struct moil_nb_params {
    double rvmx;        /* LJ cutoff (Å)                     'rvmx' */
    double relx;        /* Coulomb cutoff (Å)                'relx' */
    double eps;         /* dielectric                         'epsi' */
    double a, b, c;     /* orthorhombic box (Å)              'symm xtra ytra ztra' */
    double dtol;        /* Ewald direct-sum tolerance         'ewald dtol' (used when alpha <= 0) */
    double alpha;       /* Ewald coefficient (Å^-1); > 0 overrides dtol */
    int nfft1, nfft2, nfft3;  /* PME grid                    'grdx grdy grdz' */
    int order;          /* B-spline order                     'iord' (4 only) */
    int arith;          /* 1: Lorentz-Berthelot combination ('arith'), 0: geometric */
    int hvdw0;          /* 1 (MOIL default): geometric pairs with epsgm12 < 1e-3 are Coulomb-only */
    int lj_switch;      /* extension, not in MOIL (default 0): CHARMM LJ switch on [r_on, rvmx] */
    double r_on;
    double skin;        /* device pair-list skin (Å); lists rebuild automatically when an atom
                           moved more than skin/2 since the last build */
    int list_period;    /* > 0: also rebuild every list_period evaluations ('#lis') */
    int precision;      /* MOIL_NB_MIXED or MOIL_NB_FP64 */
} moil_nb_params;

/* Topology: the COMMON arrays of one system (borrowed; copied at init). */
typedef struct moil_topology {
    int npt;
    const double *ptchg;      /* /CONNDBL/ ptchg(npt) */
    const double *epsgm6;     /* /CONNDBL/ epsgm6(npt)  (connect/fillpt.f:136-184 encoding) */
    const double *epsgm12;    /* /CONNDBL/ epsgm12(npt) */
    const int *exc1;          /* exc1(0:npt): CSR end pointers */
    const int *exc2;          /* exc2(exc1(npt)): partner atoms, 1-based, listed under the lower atom */
    int totspe;               /* 1-4 pairs (pot/ener14.f) */
    const int *spec1, *spec2; /* 1-based */
    const double *p14;        /* p14(3,totspe): A, B, qq*kofdie*el14 */
    int totmon;
    const int *poipt;         /* poipt(totmon): last atom (1-based) of each monomer */
    const int *montype;       /* MOIL_MON_* per monomer */
} moil_topology;

/* Energies (kcal/mol), the /ENERGY/ and /EWALD3/ names eforce() fills. */
typedef struct moil_energies {
    double e_vdw, e_el;       /* primary-box LJ and real-space Coulomb */
    double e_vsym, e_lsym;    /* image (translated) LJ and real-space Coulomb */
    double e_el14, e_vdw14;   /* 1-4 */
    double e_corr;            /* exclusion erf corrections */
    double e_self;            /* Ewald self energy */
    double e_ew_receip;       /* PME reciprocal */
    double e_total;           /* sum of the above (nonbonded part of e_total) */
    double e_dir;             /* e_el + e_lsym */
} moil_energies;

/* One replica of a batch: its own parameters and topology. */
typedef struct moil_replica {
    const moil_nb_params *params;
    const moil_topology *topo;
} moil_replica;

/* Per-stage device times of the last timed evaluation (ms, CUDA events). */
typedef struct moil_nb_timing {
    float prepare_ms, list_ms, water_ms, atom_ms, excl_ms;
    float pme_spread_fft_ms, pme_conv_ms, pme_gather_ms, finalize_ms, total_ms;
    int list_rebuilt;
    int launches;             /* kernels launched by the evaluation */
} moil_nb_timing;

typedef struct moil_nb_ctx moil_nb_ctx;

/* ---- lifecycle --------------------------------------------------------- */
/* Create a handle on CUDA device `device`.  Replaces the state ewald_init()
 * and the first calls of nbondm()/syminit() set up (symm/ewald_init.f:8). */
int moil_nb_create(moil_nb_ctx **h, int device);
void moil_nb_destroy(moil_nb_ctx *h);
const char *moil_nb_strerror(int status);
const char *moil_nb_last_error(const moil_nb_ctx *h);

/* Single system: ewald_init() equivalent -- alpha (from dtol by bisection,
 * symm/ewald_init.f:298-335, unless params->alpha > 0), neutrality check,
 * self energy, B-spline moduli (pot/ewald_receip.f:413-481), topology upload. */
int moil_nb_init(moil_nb_ctx *h, const moil_nb_params *p, const moil_topology *t);

/* Batch of independent replicas (chain/path images, milestoning swarm):
 * each replica keeps its own box, cutoffs, grid and topology. */
int moil_nb_init_batch(moil_nb_ctx *h, int nrep, const moil_replica *reps);

/* Ewald coefficient the handle uses for replica r. */
int moil_nb_get_alpha(const moil_nb_ctx *h, int r, double *alpha);

/* ---- evaluation -------------------------------------------------------- */
/* Nonbonded energy + gradient of all replicas, host buffers (replica-major,
 * MOIL atom order within a replica).  dpot is overwritten with this block's
 * gradient; energies[r] per replica.  Lists rebuild as params->skin and
 * list_period require (replaces squeeze/nbondm/syminit + eforce nonbonded). */
int moil_nb_eval(moil_nb_ctx *h, const double *coor, double *dpot, moil_energies *energies);

/* The same with coordinates and gradient already in device memory
 * (device pointers, same layout); energies still go to host memory. */
int moil_nb_eval_device(moil_nb_ctx *h, const double *d_coor, double *d_dpot, moil_energies *energies);

/* moil_nb_eval_device in two halves, so the caller's host work overlaps the GPU: the first
 * queues the evaluation on the handle's streams and returns at once (after d_coor has been
 * read on the handle's stream, see moil_nb_stream, nothing orders the caller's later work);
 * the second waits for it, regrows and redoes it if a list overflowed, and returns its status
 * and energies.  One evaluation may be pending per handle: until moil_nb_eval_wait returns, the
 * caller leaves d_coor and d_dpot alone and calls nothing else on the handle but
 * moil_nb_eval_wait (other calls return MOIL_NB_ERR_STATE); moil_nb_eval_wait without a
 * pending evaluation returns MOIL_NB_ERR_STATE.  With stage timing on, the first half runs the
 * whole evaluation. */
int moil_nb_eval_device_async(moil_nb_ctx *h, const double *d_coor, double *d_dpot);
int moil_nb_eval_wait(moil_nb_ctx *h, moil_energies *energies);

/* LJ virial terms of the last evaluation for one replica, as MOIL's PRESS build accumulates
 * them into COMMON/ENERGY.BLOCK:94-96 (virvdw1..virvdw5): virvdw = -sum df1 r^2 over the
 * LJ pairs, df1 = (dE_LJ/dr)/r, for water-water pairs in the primary box
 * (pot/watwat_ewald_press.f:146-152) and across images (symm/symwat_ewald_press.f:161-168),
 * other pairs in the primary box (pot/cdie_ewald_press.f:413-419, :499-505) and across
 * images (symm/symcdie_ewald_press.f:164-167, :279-281), and 1-4 pairs
 * (pot/ener14_press.f:51-59).  dynamics/write_press.f:43-48 forms the pressure from these,
 * the constraint virial and the energies (virele = -(e_dir + e_ew_receip + e_self + e_corr)).
 * With the LJ switch extension on, df1 is the switched derivative.  On the mixed path
 * virvdw1 and virvdw2 are zero unless moil_nb_set_virial(h, 1) was called. */
int moil_nb_get_virial(moil_nb_ctx *h, int replica, double *virvdw);

/* Parameter derivatives of the nonbonded energy at coor (host, all replicas, caller order),
 * one FP64 value per atom: dE/dq (the electrostatic potential, kcal/mol/e), dE/deps and
 * dE/dsigma of the atom's LJ parameters decoded from the epsgm encoding
 * (connect/fillpt.f:136-184).  Any output may be NULL; energies as moil_nb_eval.  No
 * counterpart in the reference, which computes no parameter derivatives; both precisions
 * (pair terms in the handle's arithmetic, sums in FP64).  The LJ switch extension is not
 * differentiated. */
int moil_nb_adjoint(moil_nb_ctx *h, const double *coor, double *dEdq, double *dEdeps, double *dEdsig,
                    moil_energies *energies);

/* Force a list rebuild at the next evaluation (MOIL: nbondm() + syminit()). */
int moil_nb_request_rebuild(moil_nb_ctx *h);

/* MOIL's squeeze() on host coordinates: water and ion monomers whose first
 * atom left [-L/2, L/2] move back by one box length (symm/squeeze.f:66-145). */
int moil_nb_squeeze(const moil_nb_params *p, const moil_topology *t, double *coor);

/* Total number of atoms over all replicas. */
int moil_nb_natoms(const moil_nb_ctx *h, int64_t *natoms);

/* CUDA stream the handle launches on (cudaStream_t as void*). */
void *moil_nb_stream(const moil_nb_ctx *h);

/* ---- instrumentation --------------------------------------------------- */
int moil_nb_set_timing(moil_nb_ctx *h, int on);
int moil_nb_get_timing(const moil_nb_ctx *h, moil_nb_timing *t);
/* Pair-list entries of the last build and the unique site pairs inside the cutoff
 * predicate in the last evaluation (the pairs MOIL's kernels evaluate). */
int moil_nb_pair_stats(const moil_nb_ctx *h, int64_t *list_entries, int64_t *site_pairs);
/* Replay the device part of an evaluation as a CUDA graph (1, default) or launch
 * it kernel by kernel (0).  The graph is captured on first use and again whenever
 * the coordinate / gradient pointers or the pair-list buffers change; evaluations
 * with timing on always launch kernel by kernel.  No counterpart in the reference. */
int moil_nb_set_graph(moil_nb_ctx *h, int on);

/* ---- pressure analysis (analysis/pressure.f with pressON) ------------------ */
/* Molecules of every caller atom (all replicas back to back): mol[n] = molecule index of atom
 * n within its replica (any non-negative ids below that replica's atom count; equal ids =
 * one molecule), mass[n] = its mass (amu).  MOIL forms them in dmolecule/atom2molecule
 * (analysis/pressure.f:341-520).  mol = NULL switches the pressure terms off.  Molecules
 * are made whole by placing each atom at the minimum image of its displacement from the
 * previous atom of its molecule (consecutive atoms of a molecule must be closer than half
 * the box).  No counterpart entry point in the reference (COMMON/PRESS.BLOCK holds pmol,
 * patom and the masses). */
int moil_nb_set_molecules(moil_nb_ctx *h, const int *mol, const double *mass);
/* One evaluation of coor (moil_nb_eval semantics; dpot and energies may be NULL) and MOIL's
 * pressure analysis terms of every replica, press[12 * replica + k] =
 *   k 0..2   virXX, virYY, virZZ     LJ molecular virial (pot/watwat_ewald.f:163-175,
 *                                     pot/cdie_ewald.f:441-453, symm/symwat_ewald.f:161-173)
 *   k 3..5   V_PIdirXX..ZZ           real-space Ewald Coulomb (watwat_ewald.f:196-204)
 *   k 6..8   V_PIrecXX..ZZ           reciprocal (pot/ewald_receip.f:799-807)
 *   k 9..11  V_PIrelXX..ZZ           PME force x position relative to the centre of mass
 *                                     (ewald_receip.f:928-933)
 * in kcal/mol; pressure.f:235-238 sums vir + dir + rec - rel (its V_PIcor is zero).  Every
 * pair term is F_ij,a (R_I - R_J)_a with R the centres of mass.  Both precisions; needs
 * moil_nb_set_molecules. */
int moil_nb_pressure(moil_nb_ctx *h, const double *coor, double *dpot, moil_energies *energies, double *press);

/* Accumulate the water-water LJ virial terms (virvdw1, virvdw2 of moil_nb_get_virial) on
 * the mixed path (1), or leave them zero (0, default: the extra accumulators cost the
 * FP32 water kernel registers).  The other virial terms and the plain FP64 path always
 * accumulate them.  No counterpart in the reference (its PRESS build always does). */
int moil_nb_set_virial(moil_nb_ctx *h, int on);

/* Replica groups for the next moil_nb_init_batch: 0 automatic (three groups for batches of
 * at least a million atoms in 8 or more replicas), 1 none, P >= 2 that many.  A grouped
 * handle evaluates contiguous replica ranges concurrently, each with its own stream, lists
 * and graph, so one group's host copies and latency-bound kernels overlap another's work;
 * every replica's result is bit-identical to the ungrouped evaluation.  moil_nb_groups
 * returns the number in use.  No counterpart in the reference. */
int moil_nb_set_groups(moil_nb_ctx *h, int groups);
int moil_nb_groups(const moil_nb_ctx *h);

/* Kernel and list shapes of a handle: the search space of the autotuner
 * (moil_nb_autotune).  No counterpart in the reference, whose list scheme is fixed
 * (pot/nbondm.f:143-210, pot/nbond.f:54-157).  Every shape gives the same pair set and
 * results within the mixed path's tolerances; each is deterministic run to run. */
enum {
    MOIL_NB_WATER_AUTO = 0,       /* half lists where they apply, else full lists */
    MOIL_NB_WATER_FULL = 1,       /* one water per thread over its full row (both directions) */
    MOIL_NB_WATER_HALF = 2        /* each water pair once; the partner's share summed per block in
                                     shared memory (mixed path, replicas below 65,536 waters) */
};
enum {
    MOIL_NB_TILED_AUTO = 0,       /* all-pairs tiles where the 27-cell stencil covers >= 40% of a box */
    MOIL_NB_TILED_OFF = 1,        /* cell search for every replica */
    MOIL_NB_TILED_ALL = 2         /* all-pairs tiles for every replica of at most 16,384 waters */
};
typedef struct {
    int water_kernel;             /* MOIL_NB_WATER_* */
    int half_block;               /* waters per block of the half-list kernel: 128, 256 or 512 (0: 256) */
    int tiled;                    /* MOIL_NB_TILED_*: how the water-water rows are built */
    int groups;                   /* replica groups, as moil_nb_set_groups (next moil_nb_init_batch) */
} moil_nb_shape;

/* Set the shapes.  water_kernel, half_block and tiled apply to the current handle at once
 * (the lists are rebuilt at the next evaluation); groups applies at the next init.
 * moil_nb_get_shape returns the shapes in use, automatic choices resolved. */
int moil_nb_set_shape(moil_nb_ctx *h, const moil_nb_shape *s);
int moil_nb_get_shape(const moil_nb_ctx *h, moil_nb_shape *s);

/* One timed candidate of moil_nb_autotune. */
typedef struct {
    moil_nb_shape shape;          /* as resolved by the handle */
    double ms_per_eval;           /* wall clock per evaluation (device-resident or host buffers) */
} moil_nb_tune_trial;

/* Autotuner (no counterpart in the reference).  Times `evals` evaluations (0: one list
 * period; device-resident, or through host buffers after moil_nb_set_tune_mode) of each
 * candidate shape on the handle's batch -- the same replicas as
 * the last moil_nb_init_batch, passed again because the handle is rebuilt for each replica-
 * group count -- by coordinate descent: groups 1..4, then the water kernel (full lists, half
 * lists in blocks of 128, 256 or 512 waters), then the water-row build (automatic, cell search,
 * all-pairs tiles).  d_coor / d_dpot are device buffers of the batch.  The fastest shape
 * stays applied and is returned in *best; trials (up to max_trials, may be NULL) receive every
 * candidate timed, *ntrials their number.  With a cache file set (moil_nb_set_tune_cache) the
 * result is stored under a key made of the GPU model, its multiprocessor count, the
 * precision, the replica count and the replica-size histogram (power-of-two atom bins), and
 * moil_nb_init_batch applies a stored shape for a matching batch. */
int moil_nb_set_tune_cache(moil_nb_ctx *h, const char *path);

/* What the autotuner times: device-resident evaluations (MOIL_NB_TUNE_DEVICE, the default) or
 * evaluations through host buffers (MOIL_NB_TUNE_HOST: moil_nb_eval on page-locked copies of
 * the batch that the tuner allocates for the search), whose copies more replica groups hide
 * better.  The mode is part of the cache key. */
enum { MOIL_NB_TUNE_DEVICE = 0, MOIL_NB_TUNE_HOST = 1 };
int moil_nb_set_tune_mode(moil_nb_ctx *h, int mode);
int moil_nb_autotune(moil_nb_ctx *h, int nrep, const moil_replica *reps, const double *d_coor, double *d_dpot,
                     int evals, moil_nb_shape *best, moil_nb_tune_trial *trials, int max_trials, int *ntrials);

/* ---- PME reciprocal sum without device allocation -------------------------
 * No counterpart in the reference (MOIL's ewald_receip() works on static COMMON
 * arrays and never allocates).  This entry point is for callers that cannot call
 * cudaMalloc: a host program whose device memory is already claimed by another
 * runtime's caching pool, or code that cannot accept the device-wide
 * synchronisation that cudaMalloc/cudaFree may impose in the middle of its own
 * stream work.  It computes the PME reciprocal energy and its gradient for one
 * system with the same kernels as the handle path, taking every scratch buffer
 * from one file-scope device array of about 7.5 MB that each GPU loading this
 * library holds until the process exits.
 *   limits   natom <= 65536; each grid side 4..64 and 2/3/5-smooth; order 4;
 *            mixed precision (FP32 spline and FFT math, FP64 energy)
 *   device   d_coor (3*natom, x,y,z per atom), d_q (natom), d_dpot (3*natom,
 *            OVERWRITTEN with the reciprocal-space gradient dE/dx)
 *   host     box[3], grid[3] (nfft1..3), *e_recip (energy, kcal/mol)
 *   stream   cudaStream_t as void* (0: the default stream); the call returns after
 *            synchronising it
 * The first call on a device looks up the device address of the array (set-up) and
 * keeps it for the life of the process: resetting the device afterwards is not
 * supported.  Make that first call before any stream capture.  No call may be made on
 * a stream that is being captured into a CUDA graph: every call synchronises its
 * stream and copies the energy into host memory.  A CUDA error pending when the call
 * starts, or raised by its launches, is returned as MOIL_NB_ERR_CUDA and left pending;
 * a grid whose planes do not fit in shared memory is refused with MOIL_NB_ERR_GRID.
 * Every call reuses the same array
 * and leaves the last call's contents in it (the bin counters are cleared each call,
 * all other regions are rewritten before they are read), so calls that overlap on
 * the GPU -- from two streams or two host threads -- race: serialise them. */
int moil_nb_pme_noalloc(const double *d_coor, const double *d_q, int natom, const double *box,
                        const int *grid, double alpha, double eps, double *d_dpot, double *e_recip,
                        void *stream);

/* ---- Molecular dynamics around the evaluation (device-resident) ------------
 * nsteps leapfrog steps of the handle's system(s): each step evaluates the nonbonded
 * gradient at d_coor, then v -= dt * 418.4 * dpot / m and x += dt * v (Å, ps, amu,
 * kcal/mol), water molecules held rigid by SETTLE (Miyamoto & Kollman 1992) at the
 * distances water_geom = (O-H, H-H) (NULL: TIP3P, O-H 0.9572 and H-O-H 104.52 degrees),
 * other atoms free (the
 * library holds no bonded terms).  Stands in for dynamics/dyna.f:183-330 with SHAKE on
 * water (dynamics/shakept.f, mshakpt.f) when the nonbonded terms are the whole force field.
 *   d_coor, d_vel (3*natom, caller order, updated in place; d_vel holds v(t - dt/2) on entry
 *   and v(t + dt/2) on return), d_mass (natom), dt in ps
 *   energies: those of the last step's evaluation; *ekin: kinetic energy of the returned
 *   half-step velocities (kcal/mol), either may be NULL.  No counterpart in the reference's
 *   C/Fortran interface (its integrator stays in Fortran). */
int moil_nb_md_step(moil_nb_ctx *h, double *d_coor, double *d_vel, const double *d_mass, double dt, int nsteps,
                    const double *water_geom, moil_energies *energies, double *ekin);

/* Trajectory frames in the binary format of dynamics/wdyncrd.f (Fortran unformatted
 * sequential records): with first != 0 the file is created with the header ('CORD' + 20
 * integers, nframes in the first; a title record; the atom count) before the frame; else
 * the frame is appended.  A frame is three records of natom floats (x, y, z). */
int moil_nb_dcd_write(const char *path, int first, int nframes, int natom, const double *coor);

/* ---- Fortran entry points (gfortran naming, all arguments by reference) --
 * A maintainer replaces the nonbonded block of pot/eforce.f:122-204 with
 *     call eforce_nb_gpu(npt, coor, dpot, enb, status)
 * where enb(11) receives the moil_energies fields in declaration order.
 * The handle lives in a library-held slot set up by ewald_init_gpu; eforce_nb_gpu ADDS
 * the nonbonded gradient to dpot (MOIL's terms accumulate after eforce zeroes dpot).
 * params11 = (rvmx, relx, eps, a, b, c, dtol, alpha, r_on, skin, list_period)
 * iparams8 = (nfft1, nfft2, nfft3, order, arith, hvdw0, lj_switch, precision) */
void ewald_init_gpu_(const int *npt, const double *ptchg, const double *epsgm6, const double *epsgm12,
                     const int *exc1, const int *exc2, const int *totspe, const int *spec1, const int *spec2,
                     const double *p14, const int *totmon, const int *poipt, const int *montype,
                     const double *params11, const int *iparams8, int *status);
void nblist_gpu_(int *status);
void eforce_nb_gpu_(const int *npt, const double *coor, double *dpot, double *enb, int *status);
/* The PRESS build's eforce (pot/eforce_press.f): as eforce_nb_gpu, plus virvdw(5) =
 * virvdw1..virvdw5 of the evaluation (moil_nb_get_virial). */
void eforce_nb_press_gpu_(const int *npt, const double *coor, double *dpot, double *enb, double *virvdw,
                          int *status);

#ifdef __cplusplus
}
#endif
#endif /* MOIL_NB_H */
