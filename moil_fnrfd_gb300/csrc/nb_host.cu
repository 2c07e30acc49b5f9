// nb_host.cu -- C ABI: handle lifecycle, ewald_init equivalent, evaluation driver.
//
// An evaluation is one stream-ordered sequence with no host round trip until the final
// copy of energies and status:
//   prepare     caller FP64 coordinates -> site-ordered FP32 (or FP64) copies; sets the
//               device rebuild flag when any site moved more than skin/2 since the build
//   lists       (device-gated) unit sort + W1/W2/X list count/scan/fill
//   real space  water-molecule kernel and non-water-atom kernel
//   excl/1-4    FP64 corrections
//   PME         bin, spread+FFT(x,y), FFT(z)+convolution, FFT(y,x)+gather
//   finalize    gradient assembly in MOIL order, per-replica energies
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "nb_internal.h"

namespace {

const char *kStatusText[] = {
    "ok", "bad argument", "CUDA error", "system not neutral", "unsupported PME grid",
    "cutoff does not fit half the box", "pair-list capacity exceeded", "non-finite coordinate or result",
    "unsupported water topology", "bounded device wait expired", "out of memory", "call order"};

// symm/ewald_init.f:298-335 (find_ewaldcof): doubling, then 60+i bisection steps
double find_ewaldcof(double cutoff, double dtol)
{
    double x = 0.5, xlo, xhi;
    int i = 0;
    do {
        x *= 2.0;
        ++i;
    } while (erfc(x * cutoff) / cutoff >= dtol);
    int n = i + 60;
    xlo = 0.0;
    xhi = x;
    for (i = 1; i <= n; ++i) {
        x = 0.5 * (xlo + xhi);
        if (erfc(x * cutoff) / cutoff >= dtol) xlo = x; else xhi = x;
    }
    return x;
}

}  // namespace

// pot/ewald_receip.f:413-481 (load_bsp_moduli / DFTMOD) for order 4
void nb_bsp_moduli(int n, double *mod)
{
    // B-spline values at w = 0 (fill_bspline): 1/6, 2/3, 1/6, 0 in slots 2..5
    std::vector<double> arr(n + 8, 0.0);
    const double th[4] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 0.0};
    for (int j = 2; j <= 5 && j <= n; ++j) arr[j - 1] = th[j - 2];
    for (int k = 1; k <= n; ++k) {
        double s1 = 0, s2 = 0;
        for (int j = 1; j <= n; ++j) {
            double arg = 2.0 * M_PI * (k - 1) * (j - 1) / n;
            s1 += arr[j - 1] * cos(arg);
            s2 += arr[j - 1] * sin(arg);
        }
        mod[k - 1] = s1 * s1 + s2 * s2;
    }
    for (int k = 1; k <= n; ++k)
        if (mod[k - 1] < 1e-7) mod[k - 1] = 0.5 * (mod[(k - 2 + n) % n] + mod[k % n]);
}

namespace {

template <typename T> void free_ptr(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}

void release_device(NbCtx *c)
{
    free_ptr(c->d_reps); free_ptr(c->d_q); free_ptr(c->d_lj_f); free_ptr(c->d_lj_d); free_ptr(c->d_aflags);
    free_ptr(c->d_atom_rep); free_ptr(c->d_unit_atom); free_ptr(c->d_unit_rep); free_ptr(c->d_unit_key);
    free_ptr(c->d_unit_slot); free_ptr(c->d_bin_count); free_ptr(c->d_bin_start); free_ptr(c->d_sorted_unit);
    free_ptr(c->d_site_orig); free_ptr(c->d_site_of); free_ptr(c->d_site_rep); free_ptr(c->d_site_flags);
    free_ptr(c->d_pos); free_ptr(c->d_posb); free_ptr(c->d_woff); free_ptr(c->d_site_lj); free_ptr(c->d_site_q);
    free_ptr(c->d_wl1_cnt); free_ptr(c->d_wl1); free_ptr(c->d_wl2_off); free_ptr(c->d_wl2); free_ptr(c->d_xl_off);
    free_ptr(c->d_xl); free_ptr(c->d_count_tmp); free_ptr(c->d_ex_off); free_ptr(c->d_ex_j); free_ptr(c->d_p14_off);
    free_ptr(c->d_p14_j); free_ptr(c->d_p14_par); free_ptr(c->d_grad_site); free_ptr(c->d_e_unit);
    free_ptr(c->d_grad_ex); free_ptr(c->d_e_ex); free_ptr(c->d_plans); free_ptr(c->d_rep_plan); free_ptr(c->d_tw);
    free_ptr(c->d_tab); free_ptr(c->d_wtiles); free_ptr(c->d_scan_tmp);
    free_ptr(c->d_hblocks); free_ptr(c->d_hrow); free_ptr(c->d_hcnt); free_ptr(c->d_jset); free_ptr(c->d_jn);
    c->hblocks.clear();
    c->whalf = 0;
    free_ptr(c->d_bsp); free_ptr(c->d_etab); free_ptr(c->d_zcount); free_ptr(c->d_zstart); free_ptr(c->d_zslot); free_ptr(c->d_zatoms);
    free_ptr(c->d_fr); free_ptr(c->d_grid); free_ptr(c->d_part); free_ptr(c->d_planes); free_ptr(c->d_cols);
    free_ptr(c->d_col_begin); free_ptr(c->d_e_col); free_ptr(c->d_e_rep);
    free_ptr(c->d_echunks); free_ptr(c->d_echunk_begin); free_ptr(c->d_epart);
    c->echunks.clear(); free_ptr(c->d_coor); free_ptr(c->d_dpot);
    free_ptr(c->d_adj); free_ptr(c->d_adj_phi); free_ptr(c->d_md_dpot); free_ptr(c->d_mdctl);
    free_ptr(c->d_md_save);
    free_ptr(c->d_mol_off); free_ptr(c->d_mol_atom); free_ptr(c->d_mass); free_ptr(c->d_xrel);
    free_ptr(c->d_xsite); free_ptr(c->d_press_unit); free_ptr(c->d_press_site); free_ptr(c->d_press_col); free_ptr(c->d_press_grid);
    free_ptr(c->d_press_out);
    c->nmol = 0;
    if (c->h_e_rep) cudaFreeHost(c->h_e_rep);
    c->h_e_rep = nullptr;
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    if (c->gexec_md) cudaGraphExecDestroy(c->gexec_md);
    c->gexec_md = nullptr;
    c->inited = 0;
}

int validate_replica(NbCtx *c, const moil_nb_params *p, const moil_topology *t, int r)
{
    char buf[256];
    if (!p || !t || t->npt <= 0 || !t->ptchg || !t->epsgm6 || !t->epsgm12 || !t->exc1 || !t->poipt ||
        !t->montype || t->totmon <= 0) {
        snprintf(buf, sizeof buf, "replica %d: missing topology arrays", r);
        c->err = buf;
        return MOIL_NB_ERR_ARG;
    }
    if (t->poipt[t->totmon - 1] != t->npt) {
        snprintf(buf, sizeof buf, "replica %d: poipt(totmon) != npt", r);
        c->err = buf;
        return MOIL_NB_ERR_ARG;
    }
    double tot = 0;
    for (int i = 0; i < t->npt; ++i) tot += t->ptchg[i];
    if (fabs(tot) > 1e-7) {   // symm/ewald_init.f:62-72
        snprintf(buf, sizeof buf, "replica %d: total charge %.3e (add counterions)", r, tot);
        c->err = buf;
        return MOIL_NB_ERR_NONNEUTRAL;
    }
    if (p->order != 4) { c->err = "only spline order 4 is implemented"; return MOIL_NB_ERR_GRID; }
    double rmax = std::max(p->rvmx, p->relx);
    double lmin = std::min(p->a, std::min(p->b, p->c));
    if (!(rmax > 0) || !(lmin > 0) || rmax > 0.5 * lmin) {
        snprintf(buf, sizeof buf, "replica %d: cutoff %.3f exceeds half the box %.3f", r, rmax, 0.5 * lmin);
        c->err = buf;
        return MOIL_NB_ERR_BOX;
    }
    return MOIL_NB_OK;
}

// exclusion partner lookup in MOIL's CSR (1-based)
bool excl_has(const moil_topology *t, int l, int m)
{
    for (int k = t->exc1[l - 1] + 1; k <= t->exc1[l]; ++k)
        if (t->exc2[k - 1] == m) return true;
    return false;
}

template <typename V> int upload(NbCtx *c, V *&dst, const std::vector<V> &src)
{
    size_t n = std::max<size_t>(src.size(), 1);
    NB_CUDA_OK(c, cudaMalloc((void **)&dst, sizeof(V) * n));
    if (!src.empty()) NB_CUDA_OK(c, cudaMemcpy(dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice));
    return MOIL_NB_OK;
}

#define NB_TRY(x)                      \
    do {                               \
        int rc_ = (x);                 \
        if (rc_ != MOIL_NB_OK) return rc_; \
    } while (0)

// Water-water rows by all-pairs tiles (k_wlist_tiled) or by cell search (k_wlist).  By
// default the tiles take replicas where the 27-cell stencil already covers at least 40% of
// the box (2-4 cells per side); moil_nb_set_shape can switch them off or on everywhere.
int tiled_choice(const NbCtx *c, const RepDev &R)
{
    if (R.nwat <= 0 || R.nwat > 16384 || c->want_tiled == MOIL_NB_TILED_OFF) return 0;
    if (c->want_tiled == MOIL_NB_TILED_ALL) return 1;
    double frac = 1.0;
    for (int d = 0; d < 3; ++d) frac *= (double)std::min(R.nc[d], 3) / R.nc[d];
    return frac >= 0.4 ? 1 : 0;
}

// the tile work list of the replicas built by tiles (NB_WTILE waters per block)
int setup_tiles(NbCtx *c)
{
    free_ptr(c->d_wtiles);
    c->wtiles.clear();
    for (int r = 0; r < c->nrep; ++r) {
        const RepDev &R = c->rd[r];
        if (!R.wtiled) continue;
        for (int i0 = 0; i0 < R.nwat; i0 += NB_WTILE) c->wtiles.push_back(make_int2(r, R.wat0 + i0));
    }
    if (!c->wtiles.empty()) NB_TRY(upload(c, c->d_wtiles, c->wtiles));
    return MOIL_NB_OK;
}

// Half water rows and j-sets at the current capacities.  When the j-set of the largest
// block no longer fits the device's shared memory, the handle goes back to full lists.
int alloc_half(NbCtx *c)
{
    free_ptr(c->d_hrow);
    free_ptr(c->d_jset);
    if (!c->whalf) return MOIL_NB_OK;
    if (nb_half_configure(c) != MOIL_NB_OK || (c->want_whalf == MOIL_NB_WATER_AUTO && !nb_half_two_blocks(c))) {
        // the j-sets no longer fit (at two blocks per SM for the automatic choice): full lists
        c->whalf = 0;
        c->need_rebuild = 1;
        return MOIL_NB_OK;
    }
    const int64_t nb = (int64_t)c->hblocks.size();
    NB_CUDA_OK(c, cudaMalloc(&c->d_hrow, sizeof(unsigned) * std::max<int64_t>(nb * c->hb * c->caph, 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_jset, sizeof(int) * std::max<int64_t>(nb * c->jcap, 1)));
    return MOIL_NB_OK;
}

// Half-list set-up for the current shape: on for FP32 handles whose replicas all have fewer
// than 65,536 waters (16-bit rows) unless full lists were asked for; blocks of hb waters
// never straddle replicas.  Capacities start from the full rows and the replica sizes and
// are regrown from the build's maxima.
int setup_half(NbCtx *c)
{
    free_ptr(c->d_hblocks); free_ptr(c->d_hcnt); free_ptr(c->d_jn);
    free_ptr(c->d_hrow); free_ptr(c->d_jset);
    c->hblocks.clear();
    c->whalf = c->precision != MOIL_NB_FP64 && c->row16 && c->nW > 0 && c->want_whalf != MOIL_NB_WATER_FULL;
    if (!c->whalf) return MOIL_NB_OK;
    int maxw = 0;
    for (int r = 0; r < c->nrep; ++r) {
        const RepDev &R = c->rd[r];
        maxw = std::max(maxw, R.nwat);
        for (int i0 = 0; i0 < R.nwat; i0 += c->hb) c->hblocks.push_back(make_int2(r, R.wat0 + i0));
    }
    NB_TRY(upload(c, c->d_hblocks, c->hblocks));
    NB_CUDA_OK(c, cudaMalloc(&c->d_hcnt, sizeof(int2) * c->nW));
    NB_CUDA_OK(c, cudaMalloc(&c->d_jn, sizeof(int) * c->hblocks.size()));
    NB_CUDA_OK(c, cudaMemset(c->d_hcnt, 0, sizeof(int2) * c->nW));
    NB_CUDA_OK(c, cudaMemset(c->d_jn, 0, sizeof(int) * c->hblocks.size()));
    c->caph = ((c->cap_row1 * 5 / 8 + 32) + 31) & ~31;
    c->jcap = std::min(maxw, 7 * c->hb);
    c->need_rebuild = 1;
    return alloc_half(c);
}

// The energy reduction's fixed partition: per replica its water units, other units, atoms
// (skipped on the mixed path for a replica of waters whose corrections the water kernel adds)
// and PME column items, in chunks of NB_FE_SEG counted from the replica's own start (so a
// replica reduces in the same order alone, in a batch or in a replica group).
int setup_energy_chunks(NbCtx *c, int water_fast)
{
    c->echunks.clear();
    std::vector<int> begin(c->nrep + 1, 0);
    auto add = [&](int r, int kind, int64_t b, int64_t e) {
        for (int64_t x = b; x < e; x += NB_FE_SEG)
            c->echunks.push_back(EChunk{r, kind, (int)x, (int)std::min<int64_t>(x + NB_FE_SEG, e)});
    };
    const bool skip_ex = c->precision != MOIL_NB_FP64 && water_fast;
    for (int r = 0; r < c->nrep; ++r) {
        const RepDev &R = c->rd[r];
        begin[r] = (int)c->echunks.size();
        add(r, 0, R.wat0, (int64_t)R.wat0 + R.nwat);
        add(r, 1, c->nW + R.oth0, c->nW + (int64_t)R.oth0 + R.noth);
        if (!(skip_ex && R.noth == 0 && R.nwat > 0)) add(r, 2, R.atom0, (int64_t)R.atom0 + R.natom);
        add(r, 3, c->col_begin[r], c->col_begin[r + 1]);
    }
    begin[c->nrep] = (int)c->echunks.size();
    NB_TRY(upload(c, c->d_echunks, c->echunks));
    NB_TRY(upload(c, c->d_echunk_begin, begin));
    NB_CUDA_OK(c, cudaMalloc(&c->d_epart, sizeof(double) * NB_EU * std::max<size_t>(c->echunks.size(), 1)));
    return MOIL_NB_OK;
}

int alloc_lists(NbCtx *c)
{
    free_ptr(c->d_wl1);
    free_ptr(c->d_wl2);
    free_ptr(c->d_xl);
    const size_t entry = c->row16 ? sizeof(unsigned short) : sizeof(int);
    NB_CUDA_OK(c, cudaMalloc(&c->d_wl1, entry * std::max<int64_t>(c->nW * c->cap_row1, 2)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_wl2, sizeof(int) * std::max<int64_t>(c->cap_wl2, 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_xl, sizeof(int) * std::max<int64_t>(c->cap_xl, 1)));
    c->list_gen++;   // a captured evaluation graph refers to the old buffers
    return alloc_half(c);
}

int init_impl(NbCtx *c, int nrep, const moil_replica *reps)
{
    if (c->inited) release_device(c);
    c->err.clear();
    if (nrep <= 0 || !reps) { c->err = "no replicas"; return MOIL_NB_ERR_ARG; }
    const moil_nb_params &p0 = *reps[0].params;
    c->precision = p0.precision == MOIL_NB_FP64 ? MOIL_NB_FP64 : MOIL_NB_MIXED;
    c->skin = (float)(p0.skin > 0 ? p0.skin : 0.0);
    c->list_period = p0.list_period;
    c->nrep = nrep;
    c->rh.assign(nrep, RepHost());
    c->rd.assign(nrep, RepDev());
    c->bsp_h.clear();
    // host staging
    std::vector<double> q, lj_e12, lj_e6;
    std::vector<unsigned> aflags;
    std::vector<int> atom_rep, unit_atom_w, unit_atom_o, unit_rep_w, unit_rep_o;
    std::vector<std::vector<int>> exn, p14n;
    std::vector<std::vector<double>> p14p;
    int64_t atom0 = 0, wat0 = 0, oth0 = 0, zb0 = 0, g0 = 0;
    int water_fast = 1;
    int cell0 = 0;
    for (int r = 0; r < nrep; ++r) {
        const moil_nb_params *p = reps[r].params;
        const moil_topology *t = reps[r].topo;
        NB_TRY(validate_replica(c, p, t, r));
        if ((p->precision == MOIL_NB_FP64) != (c->precision == MOIL_NB_FP64)) {
            c->err = "all replicas of a handle must use one precision";
            return MOIL_NB_ERR_ARG;
        }
        RepHost &H = c->rh[r];
        RepDev &R = c->rd[r];
        memset(&R, 0, sizeof(R));
        H.p = *p;
        H.npt = t->npt;
        double alpha = p->alpha > 0 ? p->alpha : find_ewaldcof(p->relx, p->dtol > 0 ? p->dtol : 1e-6);
        H.alpha = alpha;
        double epstmp = NB_KOFDIE / p->eps;
        // water monomers: O,H,H with all intramolecular pairs excluded
        int nwat = 0, last_o = -1;
        std::vector<char> is_w(t->npt + 1, 0);
        for (int m = 0; m < t->totmon; ++m) {
            int first = m == 0 ? 1 : t->poipt[m - 1] + 1, last = t->poipt[m];
            if (t->montype[m] == MOIL_MON_WATER) {
                if (last - first != 2 || !excl_has(t, first, first + 1) || !excl_has(t, first, first + 2) ||
                    !excl_has(t, first + 1, first + 2)) {
                    char buf[160];
                    snprintf(buf, sizeof buf, "replica %d monomer %d: water must be O,H,H with its three pairs excluded", r, m + 1);
                    c->err = buf;
                    return MOIL_NB_ERR_TOPOLOGY;
                }
                for (int k = first; k <= last; ++k) is_w[k] = 1;
                ++nwat;
                last_o = first;
                // the per-molecule correction kernel needs exactly the three pairs, once each
                if (t->exc1[first] - t->exc1[first - 1] != 2 || t->exc1[first + 1] - t->exc1[first] != 1 ||
                    t->exc1[first + 2] - t->exc1[first + 1] != 0)
                    water_fast = 0;
            }
        }
        // exclusions: water atoms only with their own molecule
        for (int l = 1; l <= t->npt; ++l)
            for (int k = t->exc1[l - 1] + 1; k <= t->exc1[l]; ++k) {
                int m = t->exc2[k - 1];
                if (m < 1 || m > t->npt) { c->err = "exclusion partner out of range"; return MOIL_NB_ERR_ARG; }
                if ((is_w[l] || is_w[m])) {
                    bool same = is_w[l] && is_w[m] && std::abs(l - m) <= 2;
                    if (same) {
                        // same molecule iff they share the monomer (O index <= both <= O+2)
                    }
                    if (!(is_w[l] && is_w[m]) || !same) {
                        c->err = "exclusions between a water and another monomer are not supported";
                        return MOIL_NB_ERR_TOPOLOGY;
                    }
                }
            }
        // replica geometry and constants
        R.atom0 = (int)atom0; R.natom = t->npt;
        R.L[0] = (float)p->a; R.L[1] = (float)p->b; R.L[2] = (float)p->c;
        R.Ld[0] = p->a; R.Ld[1] = p->b; R.Ld[2] = p->c;
        for (int d = 0; d < 3; ++d) {
            R.invL[d] = (float)(1.0 / R.Ld[d]);
            R.invLd[d] = 1.0 / R.Ld[d];
            R.Llo[d] = (float)(R.Ld[d] - (double)R.L[d]);
        }
        double rmax = std::max(p->rvmx, p->relx);
        R.rv2 = (float)(p->rvmx * p->rvmx);
        R.re2 = (float)(p->relx * p->relx);
        R.rmax2 = (float)(rmax * rmax);
        double rl = rmax + c->skin, rlw = rl + c->rwat;
        R.rlist2 = (float)(rl * rl);
        R.rlistw2 = (float)(rlw * rlw);
        R.alpha = (float)alpha;
        R.alphad = alpha;
        R.ex2c = (float)(alpha * alpha * 1.4426950408889634);
        R.c2a = (float)(alpha * NB_TWO_OVER_SQRTPI);
        R.lj_switch = p->lj_switch ? 1 : 0;
        R.ron2 = (float)(p->r_on * p->r_on);
        if (p->lj_switch) {
            double d = p->rvmx * p->rvmx - p->r_on * p->r_on;
            R.swden = (float)(1.0 / (d * d * d));
        }
        R.arith = p->arith ? 1 : 0;
        R.hvdw0 = p->hvdw0 ? 1 : 0;
        R.epstmp = epstmp;
        R.has_water = nwat > 0;
        if (last_o > 0) {   // pot/watwat_ewald.f:40-79: constants from the last water
            int io = last_o - 1, ih = last_o;
            double qo = t->ptchg[io], qh = t->ptchg[ih];
            R.qqd[0] = epstmp * qo * qo; R.qqd[1] = epstmp * qo * qh; R.qqd[2] = epstmp * qh * qh;
            if (!p->arith) {
                R.w6d = t->epsgm6[io] * t->epsgm6[io];
                R.w12d = t->epsgm12[io] * t->epsgm12[io];
            } else {
                R.w6d = pow(t->epsgm12[io], 2) * pow(t->epsgm6[io], 6);
                R.w12d = pow(t->epsgm12[io], 2) * pow(t->epsgm6[io], 12);
            }
            for (int k = 0; k < 3; ++k) R.qq[k] = (float)R.qqd[k];
            R.w12 = (float)R.w12d; R.w6 = (float)R.w6d;
            R.w12c = R.w12 != 0.f ? (float)((R.w12d - (double)R.w12) / (double)R.w12) : 0.f;
            R.w6c = R.w6 != 0.f ? (float)((R.w6d - (double)R.w6) / (double)R.w6) : 0.f;
            // reference-water exclusion energies (k_wref) need every water to carry these charges
            R.wsame = 1;
            R.wfirst = -1;
            for (int m = 0; m < t->totmon; ++m) {
                if (t->montype[m] != MOIL_MON_WATER) continue;
                const int o = m == 0 ? 0 : t->poipt[m - 1];
                if (R.wfirst < 0) R.wfirst = (int)(atom0 + o);
                if (t->ptchg[o] != qo || t->ptchg[o + 1] != qh || t->ptchg[o + 2] != qh) R.wsame = 0;
            }
        }
        double s2 = 0;
        for (int i = 0; i < t->npt; ++i) s2 += t->ptchg[i] * t->ptchg[i];
        R.e_self = -alpha * sqrt(1.0 / M_PI) * epstmp * s2;   // symm/ewald_init.f:131-150
        // cells
        for (int d = 0; d < 3; ++d) R.nc[d] = std::max(1, (int)floor(R.Ld[d] / rlw));
        R.cell0 = cell0;
        cell0 += R.nc[0] * R.nc[1] * R.nc[2];
        // PME
        R.n1 = p->nfft1; R.n2 = p->nfft2; R.n3 = p->nfft3;
        if (R.n1 < 4 || R.n2 < 4 || R.n3 < 4) { c->err = "PME grid below 4 points"; return MOIL_NB_ERR_GRID; }
        R.n1h = R.n1 / 2 + 1;
        R.g0 = g0;
        g0 += (int64_t)R.n1h * R.n2 * R.n3;
        R.zb0 = (int)zb0;
        zb0 += R.n3;
        R.bsp0 = (int)c->bsp_h.size();
        {
            int ns[3] = {R.n1, R.n2, R.n3};
            for (int d = 0; d < 3; ++d) {
                std::vector<double> m(ns[d]);
                nb_bsp_moduli(ns[d], m.data());
                c->bsp_h.insert(c->bsp_h.end(), m.begin(), m.end());
            }
        }
        R.fcd = sqrt(epstmp);
        R.fc = (float)R.fcd;
        R.pme_gs[0] = (float)(R.fcd * R.n1 * R.invLd[0]);
        R.pme_gs[1] = (float)(R.fcd * R.n2 * R.invLd[1]);
        R.pme_gs[2] = (float)(R.fcd * R.n3 * R.invLd[2]);
        {
            double qmax = 0;
            for (int i = 0; i < t->npt; ++i) qmax = std::max(qmax, fabs(t->ptchg[i]));
            nb_spread_scale(qmax * R.fcd, &R);
        }
        R.pme_fac = M_PI * M_PI / (alpha * alpha);
        R.pivol = M_PI * p->a * p->b * p->c;
        nb_pme_fp32_consts(&R);
        {
            // the FP32 path spreads fl(fl(q) fl(fc)) per site (k_pme_bin): the reciprocal energy,
            // quadratic in the charges, is rescaled by sum (q fc)^2 / sum fl(..)^2, exact when
            // every charge has the same relative rounding (all waters: qH = -qO/2)
            double sd = 0.0, sf = 0.0;
            for (int i = 0; i < t->npt; ++i) {
                const double qd = t->ptchg[i] * R.fcd, qf = (double)((float)t->ptchg[i] * R.fc);
                sd += qd * qd;
                sf += qf * qf;
            }
            R.pme_qcorr = (sf > 0.0 ? sd / sf : 1.0) * R.spread216_corr * R.spread216_corr;
        }
        // atoms and units
        R.wat0 = (int)wat0; R.oth0 = (int)oth0;
        int noth = 0;
        for (int m = 0; m < t->totmon; ++m) {
            int first = m == 0 ? 1 : t->poipt[m - 1] + 1, last = t->poipt[m];
            if (t->montype[m] == MOIL_MON_WATER) {
                unit_atom_w.push_back((int)(atom0 + first - 1));
                unit_rep_w.push_back(r);
            } else {
                for (int k = first; k <= last; ++k) {
                    unit_atom_o.push_back((int)(atom0 + k - 1));
                    unit_rep_o.push_back(r);
                    ++noth;
                }
            }
        }
        R.nwat = nwat; R.noth = noth;
        wat0 += nwat; oth0 += noth;
        R.wtiled = tiled_choice(c, R);
        for (int i = 0; i < t->npt; ++i) {
            q.push_back(t->ptchg[i]);
            lj_e12.push_back(t->epsgm12[i]);
            lj_e6.push_back(t->epsgm6[i]);
            unsigned f = 0;
            if (fabs(t->ptchg[i]) > 1e-6) f |= SF_CHARGED;
            if (is_w[i + 1]) f |= SF_WATER;
            if (t->epsgm12[i] < 1e-3) f |= SF_HTINY;
            aflags.push_back(f);
            atom_rep.push_back(r);
        }
        // exclusion and 1-4 partners, both directions, caller indices
        size_t base = exn.size();
        exn.resize(base + t->npt);
        p14n.resize(base + t->npt);
        p14p.resize(base + t->npt);
        for (int l = 1; l <= t->npt; ++l)
            for (int k = t->exc1[l - 1] + 1; k <= t->exc1[l]; ++k) {
                int m = t->exc2[k - 1];
                exn[base + l - 1].push_back((int)(atom0 + m - 1));
                exn[base + m - 1].push_back((int)(atom0 + l - 1));
            }
        for (int k = 0; k < t->totspe; ++k) {
            int j = t->spec1[k], l = t->spec2[k];
            if (j < 1 || j > t->npt || l < 1 || l > t->npt) { c->err = "1-4 partner out of range"; return MOIL_NB_ERR_ARG; }
            if (is_w[j] || is_w[l]) water_fast = 0;
            for (int side = 0; side < 2; ++side) {
                int a = side ? l : j, b = side ? j : l;
                p14n[base + a - 1].push_back((int)(atom0 + b - 1));
                for (int d = 0; d < 3; ++d) p14p[base + a - 1].push_back(t->p14[3 * k + d]);
            }
        }
        atom0 += t->npt;
    }
    c->natom = atom0;
    c->nW = wat0;
    c->nA = oth0;
    c->row16 = 1;
    for (int r = 0; r < nrep; ++r) c->row16 &= c->rd[r].nwat < 65536;
    c->nsite = 3 * c->nW + c->nA;
    c->nunit = c->nW + c->nA;
    c->ncell = cell0;
    c->grid_elems = g0;
    c->nzbin = (int)zb0;
    if (c->nsite != c->natom) { c->err = "internal: site count"; return MOIL_NB_ERR_ARG; }
    for (int r = 0; r < nrep; ++r) c->rd[r].oth0 = c->rd[r].oth0;   // already set

    // device uploads
    NB_TRY(upload(c, c->d_q, q));
    {
        std::vector<float2> ljf(q.size());
        std::vector<double2> ljd(q.size());
        for (size_t i = 0; i < q.size(); ++i) {
            ljf[i] = make_float2((float)lj_e12[i], (float)lj_e6[i]);
            ljd[i] = make_double2(lj_e12[i], lj_e6[i]);
        }
        NB_TRY(upload(c, c->d_lj_f, ljf));
        NB_TRY(upload(c, c->d_lj_d, ljd));
    }
    NB_TRY(upload(c, c->d_aflags, aflags));
    NB_TRY(upload(c, c->d_atom_rep, atom_rep));
    {
        std::vector<int> ua(unit_atom_w), ur(unit_rep_w);
        ua.insert(ua.end(), unit_atom_o.begin(), unit_atom_o.end());
        ur.insert(ur.end(), unit_rep_o.begin(), unit_rep_o.end());
        NB_TRY(upload(c, c->d_unit_atom, ua));
        NB_TRY(upload(c, c->d_unit_rep, ur));
    }
    {
        std::vector<int> off(c->natom + 1, 0), js, poff(c->natom + 1, 0), pj;
        std::vector<double> pp;
        for (int64_t a = 0; a < c->natom; ++a) {
            off[a + 1] = off[a] + (int)exn[a].size();
            js.insert(js.end(), exn[a].begin(), exn[a].end());
            poff[a + 1] = poff[a] + (int)p14n[a].size();
            pj.insert(pj.end(), p14n[a].begin(), p14n[a].end());
            pp.insert(pp.end(), p14p[a].begin(), p14p[a].end());
        }
        NB_TRY(upload(c, c->d_ex_off, off));
        NB_TRY(upload(c, c->d_ex_j, js));
        NB_TRY(upload(c, c->d_p14_off, poff));
        NB_TRY(upload(c, c->d_p14_j, pj));
        NB_TRY(upload(c, c->d_p14_par, pp));
    }
    NB_TRY(upload(c, c->d_reps, c->rd));
    NB_TRY(setup_tiles(c));
    const size_t ts = c->precision == MOIL_NB_FP64 ? 8 : 4;
    int64_t nu = c->nunit, ns = c->nsite;
    NB_CUDA_OK(c, cudaMalloc(&c->d_unit_key, sizeof(int) * nu));
    NB_CUDA_OK(c, cudaMalloc(&c->d_unit_slot, sizeof(int) * nu));
    NB_CUDA_OK(c, cudaMalloc(&c->d_bin_count, sizeof(int) * (2 * c->ncell + 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_bin_start, sizeof(int) * (2 * c->ncell + 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_sorted_unit, sizeof(int) * nu));
    NB_CUDA_OK(c, cudaMalloc(&c->d_site_orig, sizeof(int) * ns));
    NB_CUDA_OK(c, cudaMemset(c->d_site_orig, 0, sizeof(int) * ns));   // valid indices before the first build
    NB_CUDA_OK(c, cudaMalloc(&c->d_site_of, sizeof(int) * ns));
    NB_CUDA_OK(c, cudaMemset(c->d_site_of, 0, sizeof(int) * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_site_rep, sizeof(int) * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_site_flags, sizeof(unsigned) * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_pos, 4 * ts * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_posb, sizeof(float4) * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_woff, 4 * ts * 3 * std::max<int64_t>(c->nW, 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_site_lj, 2 * ts * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_site_q, ts * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_wl1_cnt, sizeof(int2) * std::max<int64_t>(c->nW, 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_wl2_off, sizeof(int) * (c->nW + 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_xl_off, sizeof(int) * (c->nA + 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_count_tmp, sizeof(int) * (3 * std::max(c->nW, c->nA) + 3)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_grad_site, sizeof(long long) * 3 * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_e_unit, sizeof(double) * NB_EU * std::max<int64_t>(nu, 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_grad_ex, sizeof(double) * 3 * c->natom));
    NB_CUDA_OK(c, cudaMalloc(&c->d_e_ex, sizeof(double) * NB_EX * c->natom));
    NB_CUDA_OK(c, cudaMalloc(&c->d_zcount, sizeof(int) * (c->nzbin + 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_zstart, sizeof(int) * (c->nzbin + 1)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_zslot, sizeof(int) * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_zatoms, sizeof(int) * ns));
    NB_CUDA_OK(c, cudaMalloc(&c->d_e_rep, sizeof(double) * NB_EREP * nrep));
    NB_CUDA_OK(c, cudaMalloc(&c->d_coor, sizeof(double) * 3 * c->natom));
    NB_CUDA_OK(c, cudaMalloc(&c->d_dpot, sizeof(double) * 3 * c->natom));
    NB_CUDA_OK(c, cudaMemset(c->d_grad_site, 0, sizeof(long long) * 3 * ns));
    NB_CUDA_OK(c, cudaMemset(c->d_e_unit, 0, sizeof(double) * NB_EU * std::max<int64_t>(nu, 1)));
    // the mixed path never writes the water atoms' entries (their corrections are in the
    // water kernel): they stay zero
    NB_CUDA_OK(c, cudaMemset(c->d_grad_ex, 0, sizeof(double) * 3 * c->natom));
    NB_CUDA_OK(c, cudaMemset(c->d_e_ex, 0, sizeof(double) * NB_EX * c->natom));
    // list capacities from densities (grown on overflow)
    c->cap_wl2 = c->cap_xl = 64;
    double row1 = 32;
    for (int r = 0; r < nrep; ++r) {
        const RepDev &R = c->rd[r];
        double vol = R.Ld[0] * R.Ld[1] * R.Ld[2];
        double rl = sqrt((double)R.rlist2), rlw = sqrt((double)R.rlistw2);
        double sph = 4.0 / 3.0 * M_PI, vl = std::min(sph * rl * rl * rl, vol), vw = std::min(sph * rlw * rlw * rlw, vol);
        if (R.nwat > 0) row1 = std::max(row1, vl * R.nwat / vol * 1.4 + 32);
        c->cap_wl2 += (int64_t)(R.nwat * (vw * R.noth / vol) * 1.5) + 32;
        c->cap_xl += (int64_t)(R.noth * (vw * (3.0 * R.nwat + R.noth) / vol) * 1.5) + 32;
    }
    c->cap_row1 = ((int)row1 + 31) & ~31;
    NB_TRY(alloc_lists(c));
    NB_TRY(nb_realspace_configure(c));
    NB_TRY(setup_half(c));
    NB_CUDA_OK(c, cudaMallocHost(&c->h_e_rep, sizeof(double) * NB_EREP * nrep));
    memset(c->h_e_rep, 0, sizeof(double) * NB_EREP * nrep);
    NB_TRY(nb_pme_configure(c));
    NB_TRY(setup_energy_chunks(c, water_fast));
    {
        // tile sums for every scan: bins, per-water and per-atom counts, PME z-bins
        int64_t nmax = std::max<int64_t>({2 * (int64_t)c->ncell, c->nW, c->nA, (int64_t)c->nzbin, 1});
        NB_CUDA_OK(c, cudaMalloc(&c->d_scan_tmp, sizeof(long long) * (nmax / 4096 + 2)));
    }
    NB_CUDA_OK(c, cudaDeviceSynchronize());
    c->need_rebuild = 1;
    c->evals_since_build = 0;
    c->water_excl_fast = water_fast;
    c->inited = 1;
    return MOIL_NB_OK;
}

// While an evaluation is captured: the list rebuild goes into the body of a conditional IF
// node that a one-thread kernel sets from the device rebuild flag, so evaluations without a
// rebuild launch none of the rebuild kernels.  Returns false (the gated kernels are then
// captured in line) if the stream is not capturing or a graph call fails before the node is
// added.
bool enqueue_lists_conditional(NbCtx *c, const double *d_coor)
{
    cudaStream_t s = c->stream;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return false;
    cudaGraphConditionalHandle hc;
    if (cudaGraphConditionalHandleCreate(&hc, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return false;
    if (!c->sbody && cudaStreamCreateWithFlags(&c->sbody, cudaStreamNonBlocking) != cudaSuccess) {
        c->sbody = nullptr;
        return false;
    }
    nb_launch_rebuild_cond(c, hc);
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess) return false;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hc;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &np) != cudaSuccess) return false;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(c->sbody, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess) {
        // an empty body: the gated kernels are captured after the node instead
        cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        return false;
    }
    std::swap(c->stream, c->sbody);
    nb_launch_build_lists(c, d_coor);
    std::swap(c->stream, c->sbody);
    cudaGraph_t done = nullptr;
    cudaStreamEndCapture(c->sbody, &done);
    // the rest of the evaluation follows the conditional node (errors surface at EndCapture)
    cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    return true;
}

// The device part of one evaluation, in stream order.  The sequence does not depend on host
// state beyond the handle's fixed buffers and the two caller pointers: the rebuild decision
// travels through the pinned word h_status[8], read by the first copy.  That makes it
// capturable as a CUDA graph.
// The evaluation between its status words: coordinate preparation, list rebuild, pair, PME
// and correction kernels, gradient and energy assembly.
void enqueue_core(NbCtx *c, const double *d_coor, double *d_dpot)
{
    cudaStream_t s = c->stream;
    nb_launch_prepare(c, d_coor, 1);   // sets the rebuild flag when a site moved > skin/2
    // every rebuild kernel is gated by the flag; a captured evaluation also skips their
    // launches through a conditional node
    if (c->timing) {
        // stage timing (kernel by kernel): the host reads the flag and launches the rebuild
        // only when it is set, as the conditional node of a replayed evaluation does.  The
        // preparation stage (status upload, coordinate conversion with the skin check) ends
        // before the read-back; the rebuild stage starts after the host's decision, so
        // neither counts the round trip a replayed evaluation does not make
        cudaEventRecord(c->ev[12], s);
        cudaMemcpyAsync(c->h_status + 16, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        cudaEventRecord(c->ev[13], s);
        if (c->h_status[16]) nb_launch_build_lists(c, d_coor);
        cudaEventRecord(c->ev[1], s);
    } else if (!(c->capturing && !c->on_prio && enqueue_lists_conditional(c, d_coor))) {
        // (on the prioritised streams of host-buffer group evaluations the conditional node
        // cost the copy/kernel overlap more than the skipped launches save: gated kernels)
        nb_launch_build_lists(c, d_coor);
    }
    if (c->timing) {
        // stage timing: one stream, stage after stage
        nb_launch_realspace(c);
        nb_launch_excl14(c, d_coor);
        cudaEventRecord(c->ev[5], s);
        nb_launch_pme(c);
    } else {
        // the PME branch (binning, planes, columns, gather) runs on a second stream beside the
        // pair and correction kernels: they read the same site positions and write disjoint
        // outputs, and the latency-bound plane kernels fill the multiprocessors the pair
        // kernel leaves idle
        cudaEventRecord(c->ev_fork, s);
        cudaStreamWaitEvent(c->stream2, c->ev_fork, 0);
        std::swap(c->stream, c->stream2);
        nb_launch_pme(c);
        std::swap(c->stream, c->stream2);
        cudaEventRecord(c->ev_join, c->stream2);
        nb_launch_realspace(c);
        nb_launch_excl14(c, d_coor);
        cudaStreamWaitEvent(s, c->ev_join, 0);
    }
    nb_launch_finalize(c, d_dpot);
}

void enqueue_eval(NbCtx *c, const double *d_coor, double *d_dpot)
{
    cudaStream_t s = c->stream;
    c->launches = 0;
    if (c->timing) cudaEventRecord(c->ev[0], s);
    cudaMemcpyAsync(c->d_status, c->h_status + 8, sizeof(int) * 8, cudaMemcpyHostToDevice, s);
    enqueue_core(c, d_coor, d_dpot);
    if (c->timing) cudaEventRecord(c->ev[10], s);
    cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int) * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(c->h_e_rep, c->d_e_rep, sizeof(double) * NB_EREP * c->nrep, cudaMemcpyDeviceToHost, s);
}

// one whole MD step of a context, as captured into its step graph: a gate kernel sets an IF
// node that runs the step only while no error has been raised in the call; the step is the
// step-control kernel, the evaluation, the error bits and rebuild counter, the leapfrog +
// SETTLE integrator.  Returns false if the gate could not be built (nothing captured then).
bool enqueue_md_step(NbCtx *c, double *coor, double *vel, const double *mass, double *dpot, double dt, double doh,
                     double dhh)
{
    cudaStream_t s = c->stream;
    c->launches = 0;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return false;
    cudaGraphConditionalHandle hc;
    if (cudaGraphConditionalHandleCreate(&hc, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return false;
    if (!c->sstep && cudaStreamCreateWithFlags(&c->sstep, cudaStreamNonBlocking) != cudaSuccess) {
        c->sstep = nullptr;
        return false;
    }
    nb_launch_md_gate(c, s, hc);
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess) return false;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hc;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &np) != cudaSuccess) return false;
    if (cudaStreamBeginCaptureToGraph(c->sstep, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return false;
    std::swap(c->stream, c->sstep);
    nb_launch_md_begin(c, c->stream);
    enqueue_core(c, coor, dpot);
    nb_launch_md_end(c, c->stream);
    nb_launch_integrate(c, c->stream, coor, vel, mass, dpot, dt, doh, dhh);
    std::swap(c->stream, c->sstep);
    cudaGraph_t done = nullptr;
    cudaStreamEndCapture(c->sstep, &done);
    cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    return true;
}

void drop_graph(NbCtx *c)
{
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    if (c->gexec_md) cudaGraphExecDestroy(c->gexec_md);
    c->gexec_md = nullptr;
}

// replay the captured evaluation, capturing it first when the caller pointers or the list
// buffers changed; returns false (graph mode switched off) if capture is not possible
bool launch_graph(NbCtx *c, const double *d_coor, double *d_dpot)
{
    cudaStream_t s = c->stream;
    if (!c->gexec || c->g_coor != d_coor || c->g_dpot != d_dpot || c->g_gen != c->list_gen ||
        c->g_prio != c->on_prio) {
        drop_graph(c);
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            c->use_graph = 0;
            return false;
        }
        c->capturing = 1;
        enqueue_eval(c, d_coor, d_dpot);
        c->capturing = 0;
        cudaError_t e1 = cudaStreamEndCapture(s, &g);
        cudaError_t e2 = e1 == cudaSuccess ? cudaGraphInstantiate(&c->gexec, g, 0) : e1;
        if (g) cudaGraphDestroy(g);
        if (e2 != cudaSuccess) {
            cudaGetLastError();
            c->gexec = nullptr;
            c->use_graph = 0;
            return false;
        }
        c->g_coor = d_coor;
        c->g_dpot = d_dpot;
        c->g_prio = c->on_prio;
        c->g_gen = c->list_gen;
        c->graph_launches = c->launches;
    }
    c->launches = c->graph_launches;
    return cudaGraphLaunch(c->gexec, s) == cudaSuccess;
}

// queue one evaluation on the context's stream (no synchronisation)
void eval_launch(NbCtx *c, const double *d_coor, double *d_dpot)
{
    bool forced = c->need_rebuild || (c->list_period > 0 && c->evals_since_build >= c->list_period);
    c->h_status[8] = forced ? 1 : 0;
    for (int k = 9; k < 16; ++k) c->h_status[k] = 0;
    if (!(c->use_graph && !c->timing && launch_graph(c, d_coor, d_dpot))) enqueue_eval(c, d_coor, d_dpot);
}

// wait for the queued evaluation and read its status words
int eval_complete(NbCtx *c)
{
    NB_CUDA_OK(c, cudaStreamSynchronize(c->stream));
    NB_CUDA_OK(c, cudaGetLastError());
    int rebuilt = c->h_status[0] != 0;
    if (rebuilt) {
        c->evals_since_build = 0;
        c->last_water_pairs = c->h_status[2];
        c->last_atom_pairs = c->h_status[4];
        c->last_list_entries = (int64_t)c->h_status[2] + c->h_status[3] + c->h_status[4];
    }
    c->evals_since_build++;
    c->need_rebuild = 0;
    if (c->timing) {
        moil_nb_timing &t = c->last_timing;
        auto el = [&](int a, int b) {
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]);
            return ms;
        };
        t.prepare_ms = el(0, 12);
        t.list_ms = el(13, 1);
        t.water_ms = el(2, 3);
        t.atom_ms = el(3, 4);
        t.excl_ms = el(4, 5);
        t.pme_spread_fft_ms = el(6, 7);
        t.pme_conv_ms = el(7, 8);
        t.pme_gather_ms = el(8, 9);
        t.finalize_ms = el(9, 10);
        t.total_ms = el(0, 10);
        t.list_rebuilt = rebuilt;
        t.launches = c->launches;
    }
    int err = c->h_status[1];
    if (err & NB_DEV_ERR_OVERFLOW) return MOIL_NB_ERR_OVERFLOW;
    if (err & NB_DEV_ERR_NAN) { c->err = "non-finite coordinate or gradient"; return MOIL_NB_ERR_NAN; }
    if (err & NB_DEV_ERR_RWAT) { c->err = "a water hydrogen moved more than 1.1 A from its oxygen"; return MOIL_NB_ERR_TOPOLOGY; }
    return MOIL_NB_OK;
}

int eval_once(NbCtx *c, const double *d_coor, double *d_dpot)
{
    eval_launch(c, d_coor, d_dpot);
    return eval_complete(c);
}

// per-replica energies and the pair count of the last completed evaluation
void read_energies(NbCtx *c, moil_energies *e)
{
    if (e) {
        for (int r = 0; r < c->nrep; ++r) {
            const double *o = c->h_e_rep + NB_EREP * r;
            moil_energies &E = e[r];
            E.e_vdw = o[0]; E.e_el = o[1]; E.e_vsym = o[2]; E.e_lsym = o[3];
            E.e_el14 = o[4]; E.e_vdw14 = o[5]; E.e_corr = o[6]; E.e_self = o[7];
            E.e_ew_receip = o[8]; E.e_total = o[9]; E.e_dir = o[10];
        }
    }
    double np = 0;
    for (int r = 0; r < c->nrep; ++r) np += c->h_e_rep[NB_EREP * r + 11];
    c->last_site_pairs = (int64_t)(np + 0.5);
}

// an evaluation whose first attempt (if any) has completed with status rc: on a list
// overflow, grow the lists from the counts and redo
int eval_retry(NbCtx *c, const double *d_coor, double *d_dpot, moil_energies *e, int rc, bool done)
{
    for (int attempt = 0; attempt < 4; ++attempt) {
        if (!done || attempt > 0) rc = eval_once(c, d_coor, d_dpot);
        if (rc != MOIL_NB_ERR_OVERFLOW) break;
        // grow from the exact totals the count pass produced, then redo with a fresh build
        int64_t need1 = c->h_status[6], need2 = c->h_status[3], need3 = c->h_status[4];
        c->cap_row1 = std::max<int>(c->cap_row1, (int)((need1 + need1 / 8 + 32 + 31) & ~31));
        c->cap_wl2 = std::max<int64_t>(c->cap_wl2, need2 + need2 / 8 + 64);
        c->cap_xl = std::max<int64_t>(c->cap_xl, need3 + need3 / 8 + 64);
        if (c->whalf) {
            const int64_t needj = c->h_status[5], needh = c->h_status[7];
            c->caph = std::max<int>(c->caph, (int)((needh + needh / 8 + 32 + 31) & ~31));
            c->jcap = std::max<int>(c->jcap, (int)std::min<int64_t>(needj + needj / 8 + 64, 65535));
        }
        int a = alloc_lists(c);
        if (a != MOIL_NB_OK) return a;
        c->need_rebuild = 1;
        done = false;
    }
    if (rc != MOIL_NB_OK) return rc;
    read_energies(c, e);
    return MOIL_NB_OK;
}

int eval_impl(NbCtx *c, const double *d_coor, double *d_dpot, moil_energies *e)
{
    return eval_retry(c, d_coor, d_dpot, e, MOIL_NB_OK, false);
}

// ---- replica groups ------------------------------------------------------------------
// A large batch is split into contiguous replica ranges, each a complete context with its own
// stream, lists, PME work and graph.  The groups' evaluations are queued together and run
// concurrently: one group's host copies overlap another's kernels, and one group's
// latency-bound PME kernels share the multiprocessors with another's pair kernel.  Every
// replica's result is computed by the same kernels in the same order as without groups.
int group_of(const NbCtx *h, int r)
{
    int g = 0;
    while (g + 1 < (int)h->grp.size() && h->grp_rep0[g + 1] <= r) ++g;
    return g;
}

// phase 1 queues the groups' evaluations, phase 2 completes them (3: both)
int eval_groups(NbCtx *h, const double *coor, double *dpot, moil_energies *e, bool host, int phase = 3)
{
    const int P = (int)h->grp.size();
    // device-resident callers may have queued their coordinates on the handle's stream
    NB_CUDA_OK(h, cudaEventRecord(h->ev[11], h->stream));
    auto slice_bytes = [&](int g) { return sizeof(double) * 3 * (size_t)(h->grp_atom0[g + 1] - h->grp_atom0[g]); };
    auto launch = [&](int g) -> int {
        NbCtx *c = h->grp[g];
        NB_CUDA_OK(c, cudaStreamWaitEvent(c->stream, h->ev[11], 0));
        const double *src = coor + 3 * h->grp_atom0[g];
        double *dst = dpot + 3 * h->grp_atom0[g];
        if (host) {
            NB_CUDA_OK(c, cudaMemcpyAsync(c->d_coor, src, slice_bytes(g), cudaMemcpyHostToDevice, c->stream));
            eval_launch(c, c->d_coor, c->d_dpot);
            NB_CUDA_OK(c, cudaMemcpyAsync(dst, c->d_dpot, slice_bytes(g), cudaMemcpyDeviceToHost, c->stream));
        } else {
            eval_launch(c, src, dst);
        }
        return MOIL_NB_OK;
    };
    auto finish = [&](int g) -> int {
        NbCtx *c = h->grp[g];
        const double *dc = host ? c->d_coor : coor + 3 * h->grp_atom0[g];
        double *dd = host ? c->d_dpot : dpot + 3 * h->grp_atom0[g];
        const int first = eval_complete(c);
        int rc = eval_retry(c, dc, dd, e ? e + h->grp_rep0[g] : nullptr, first, true);
        if (rc == MOIL_NB_OK && host && first == MOIL_NB_ERR_OVERFLOW) {
            // redone after an overflow: the gradient copied with the first attempt is stale
            NB_CUDA_OK(c, cudaMemcpyAsync(dpot + 3 * h->grp_atom0[g], c->d_dpot, slice_bytes(g),
                                          cudaMemcpyDeviceToHost, c->stream));
            NB_CUDA_OK(c, cudaStreamSynchronize(c->stream));
        }
        return rc;
    };
    // host-buffer evaluations run on the prioritised streams (the graphs replay on any stream)
    auto use_prio = [&](bool on) {
        if (!host) return;
        for (NbCtx *c : h->grp)
            if (c->pstream) {
                std::swap(c->stream, c->pstream);
                std::swap(c->stream2, c->pstream2);
                c->on_prio = on ? 1 : 0;
            }
    };
    use_prio(true);
    int rc = MOIL_NB_OK;
    if (h->timing) {
        // diagnostic mode: one group after the other, stage times summed
        moil_nb_timing sum{};
        for (int g = 0; g < P && rc == MOIL_NB_OK; ++g) {
            rc = launch(g);
            if (rc == MOIL_NB_OK) rc = finish(g);
            const moil_nb_timing &t = h->grp[g]->last_timing;
            sum.prepare_ms += t.prepare_ms; sum.list_ms += t.list_ms; sum.water_ms += t.water_ms;
            sum.atom_ms += t.atom_ms; sum.excl_ms += t.excl_ms; sum.pme_spread_fft_ms += t.pme_spread_fft_ms;
            sum.pme_conv_ms += t.pme_conv_ms; sum.pme_gather_ms += t.pme_gather_ms;
            sum.finalize_ms += t.finalize_ms; sum.total_ms += t.total_ms;
            sum.list_rebuilt |= t.list_rebuilt; sum.launches += t.launches;
        }
        h->last_timing = sum;
    } else {
        if (phase & 1)
            for (int g = 0; g < P && rc == MOIL_NB_OK; ++g) rc = launch(g);
        if (phase == 1) {
            use_prio(false);
            return rc;
        }
        for (int g = 0; g < P; ++g) {
            int r = finish(g);
            if (r != MOIL_NB_OK && rc == MOIL_NB_OK) rc = r;
        }
    }
    use_prio(false);
    int64_t pairs = 0, entries = 0;
    int launches = 0;
    for (NbCtx *c : h->grp) {
        pairs += c->last_site_pairs;
        entries += c->last_list_entries;
        launches += c->launches;
        if (!c->err.empty() && h->err.empty()) h->err = c->err;
    }
    h->last_site_pairs = pairs;
    h->last_list_entries = entries;
    h->launches = launches;
    return rc;
}

std::mutex g_fortran_mu;
moil_nb_ctx *g_fortran_ctx = nullptr;
std::vector<double> g_fortran_buf;

}  // namespace

namespace {

void destroy_groups(NbCtx *h)
{
    for (NbCtx *c : h->grp) moil_nb_destroy(static_cast<moil_nb_ctx *>(c));
    h->grp.clear();
    h->grp_rep0.clear();
    h->grp_atom0.clear();
}

// groups for a batch: automatic for batches of at least a million atoms in 8 or more
// replicas (three groups), where copy/kernel overlap pays; none for smaller ones
int choose_groups(const NbCtx *h, int nrep, int64_t natom)
{
    if (h->want_groups == 1 || nrep < 2) return 1;
    if (h->want_groups >= 2) return std::min(h->want_groups, nrep);
    return (nrep >= 8 && natom >= 1000000) ? 3 : 1;
}

int init_groups(moil_nb_ctx *h, int nrep, const moil_replica *reps, int P)
{
    int64_t total = 0;
    for (int r = 0; r < nrep; ++r) total += reps[r].topo ? reps[r].topo->npt : 0;
    // contiguous replica ranges; with three or more groups the first and the last hold half
    // the atoms of the others (their host copies are the ones no kernel work hides)
    std::vector<double> cut(P + 1, 0.0);
    for (int g = 0; g < P; ++g) cut[g + 1] = cut[g] + ((P >= 3 && (g == 0 || g == P - 1)) ? 1.0 : 2.0);
    h->grp_rep0.assign(1, 0);
    h->grp_atom0.assign(1, 0);
    int64_t acc = 0;
    for (int r = 0; r < nrep; ++r) {
        acc += reps[r].topo->npt;
        const int g = (int)h->grp_rep0.size();
        if (g < P && r + 1 < nrep && (double)acc >= (double)total * cut[g] / cut[P]) {
            h->grp_rep0.push_back(r + 1);
            h->grp_atom0.push_back(acc);
        }
    }
    h->grp_rep0.push_back(nrep);
    h->grp_atom0.push_back(total);
    for (size_t g = 0; g + 1 < h->grp_rep0.size(); ++g) {
        moil_nb_ctx *c = nullptr;
        int rc = moil_nb_create(&c, h->device);
        if (rc != MOIL_NB_OK) { h->err = "creating a replica group"; destroy_groups(h); return rc; }
        c->use_graph = h->use_graph;
        c->virial = h->virial;
        c->timing = h->timing;
        c->want_whalf = h->want_whalf;
        c->hb = h->hb;
        c->want_tiled = h->want_tiled;
        {
            // streams for host-buffer evaluations: earlier groups at higher priority finish
            // first, so their gradient copies overlap the later groups' kernels (device-
            // resident evaluations keep equal priorities, which balances the kernels best)
            int lo = 0, hi = 0;
            cudaDeviceGetStreamPriorityRange(&lo, &hi);
            const int prio = std::min(lo, hi + (int)g);
            if (cudaStreamCreateWithPriority(&c->pstream, cudaStreamNonBlocking, prio) != cudaSuccess ||
                cudaStreamCreateWithPriority(&c->pstream2, cudaStreamNonBlocking, prio) != cudaSuccess) {
                h->err = "creating replica group streams";
                h->grp.push_back(c);
                destroy_groups(h);
                return MOIL_NB_ERR_CUDA;
            }
        }
        h->grp.push_back(c);
        rc = init_impl(c, h->grp_rep0[g + 1] - h->grp_rep0[g], reps + h->grp_rep0[g]);
        if (rc != MOIL_NB_OK) { h->err = c->err; destroy_groups(h); return rc; }
    }
    h->nrep = nrep;
    h->natom = total;
    h->precision = h->grp[0]->precision;
    h->inited = 1;
    return MOIL_NB_OK;
}

}  // namespace

extern "C" {

const char *moil_nb_strerror(int s)
{
    if (s < 0 || s >= (int)(sizeof(kStatusText) / sizeof(kStatusText[0]))) return "unknown status";
    return kStatusText[s];
}

const char *moil_nb_last_error(const moil_nb_ctx *h) { return h ? h->err.c_str() : "null handle"; }

int moil_nb_create(moil_nb_ctx **out, int device)
{
    if (!out) return MOIL_NB_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return MOIL_NB_ERR_CUDA;
    if (device < 0 || device >= ndev) return MOIL_NB_ERR_ARG;
    moil_nb_ctx *h = new moil_nb_ctx();
    h->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        if (h->stream) cudaStreamDestroy(h->stream);
        if (h->stream2) cudaStreamDestroy(h->stream2);
        if (h->ev_fork) cudaEventDestroy(h->ev_fork);
        delete h;
        return MOIL_NB_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, device);
    if (h->nsm <= 0) h->nsm = 1;
    for (int k = 0; k < NB_NEV; ++k) cudaEventCreate(&h->ev[k]);
    if (cudaMallocHost(&h->h_status, sizeof(int) * 24) != cudaSuccess || cudaMalloc(&h->d_status, sizeof(int) * 8) != cudaSuccess) {
        moil_nb_destroy(h);
        return MOIL_NB_ERR_CUDA;
    }
    cudaMemset(h->d_status, 0, sizeof(int) * 8);
    *out = h;
    return MOIL_NB_OK;
}

void moil_nb_destroy(moil_nb_ctx *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    destroy_groups(h);
    release_device(h);
    for (int k = 0; k < NB_NEV; ++k)
        if (h->ev[k]) cudaEventDestroy(h->ev[k]);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->d_status) cudaFree(h->d_status);
    if (h->stream2) { cudaStreamSynchronize(h->stream2); cudaStreamDestroy(h->stream2); }
    if (h->sbody) cudaStreamDestroy(h->sbody);
    if (h->sstep) cudaStreamDestroy(h->sstep);
    if (h->pstream) cudaStreamDestroy(h->pstream);
    if (h->pstream2) cudaStreamDestroy(h->pstream2);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int moil_nb_init(moil_nb_ctx *h, const moil_nb_params *p, const moil_topology *t)
{
    if (!h || !p || !t) return MOIL_NB_ERR_ARG;
    moil_replica r = {p, t};
    cudaSetDevice(h->device);
    destroy_groups(h);
    return init_impl(h, 1, &r);
}

int moil_nb_init_batch(moil_nb_ctx *h, int nrep, const moil_replica *reps)
{
    if (!h) return MOIL_NB_ERR_ARG;
    if (h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    destroy_groups(h);
    int64_t natom = 0;
    for (int r = 0; r < nrep && reps; ++r) {
        if (!reps[r].params || !reps[r].topo) { h->err = "replica without parameters or topology"; return MOIL_NB_ERR_ARG; }
        natom += reps[r].topo->npt;
    }
    if (reps) nb_tune_cached_shape(h, nrep, reps);
    const int P = reps ? choose_groups(h, nrep, natom) : 1;
    if (P <= 1) return init_impl(h, nrep, reps);
    if (h->inited) release_device(h);
    h->inited = 0;
    return init_groups(h, nrep, reps, P);
}

int moil_nb_get_alpha(const moil_nb_ctx *h, int r, double *alpha)
{
    if (!h || !alpha || !h->inited || r < 0 || r >= h->nrep) return MOIL_NB_ERR_ARG;
    if (!h->grp.empty()) {
        const int g = group_of(h, r);
        return moil_nb_get_alpha(static_cast<const moil_nb_ctx *>(h->grp[g]), r - h->grp_rep0[g], alpha);
    }
    *alpha = h->rh[r].alpha;
    return MOIL_NB_OK;
}

int moil_nb_eval(moil_nb_ctx *h, const double *coor, double *dpot, moil_energies *e)
{
    if (!h || !coor || !dpot) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    if (!h->grp.empty()) return eval_groups(h, coor, dpot, e, true);
    // staged through device copies even for pinned buffers: on GB300 the finalize kernel
    // storing 63 MB of gradient straight into pinned host memory took 1.15 ms, while copying
    // the coordinates in and the gradient out took 0.7 ms together
    size_t bytes = sizeof(double) * 3 * h->natom;
    NB_CUDA_OK(h, cudaMemcpyAsync(h->d_coor, coor, bytes, cudaMemcpyHostToDevice, h->stream));
    int rc = eval_impl(h, h->d_coor, h->d_dpot, e);
    if (rc != MOIL_NB_OK) return rc;
    NB_CUDA_OK(h, cudaMemcpyAsync(dpot, h->d_dpot, bytes, cudaMemcpyDeviceToHost, h->stream));
    NB_CUDA_OK(h, cudaStreamSynchronize(h->stream));
    return MOIL_NB_OK;
}

int moil_nb_adjoint(moil_nb_ctx *h, const double *coor, double *dEdq, double *dEdeps, double *dEdsig,
                    moil_energies *e)
{
    if (!h || !coor) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    if (!h->grp.empty()) {
        for (size_t g = 0; g < h->grp.size(); ++g) {
            const int64_t a0 = h->grp_atom0[g];
            auto at = [&](double *p) { return p ? p + a0 : nullptr; };
            int rc = moil_nb_adjoint(static_cast<moil_nb_ctx *>(h->grp[g]), coor + 3 * a0, at(dEdq), at(dEdeps),
                                     at(dEdsig), e ? e + h->grp_rep0[g] : nullptr);
            if (rc != MOIL_NB_OK) { h->err = h->grp[g]->err; return rc; }
        }
        return MOIL_NB_OK;
    }
    const size_t n = (size_t)h->natom;
    NB_CUDA_OK(h, cudaMemcpyAsync(h->d_coor, coor, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream));
    int rc = eval_impl(h, h->d_coor, h->d_dpot, e);   // lists, positions and the potential grid
    if (rc != MOIL_NB_OK) return rc;
    if (!h->d_adj) NB_CUDA_OK(h, cudaMalloc(&h->d_adj, sizeof(double) * 3 * std::max<size_t>(n, 1)));
    if (h->precision == MOIL_NB_FP64 && !h->d_adj_phi)
        NB_CUDA_OK(h, cudaMalloc(&h->d_adj_phi, sizeof(double) * 4 * std::max<int64_t>(h->nsite, 1)));
    rc = nb_adjoint(h, h->d_adj, h->d_adj + n, h->d_adj + 2 * n);
    if (rc != MOIL_NB_OK) return rc;
    double *out[3] = {dEdq, dEdeps, dEdsig};
    for (int k = 0; k < 3; ++k)
        if (out[k])
            NB_CUDA_OK(h, cudaMemcpyAsync(out[k], h->d_adj + k * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                          h->stream));
    NB_CUDA_OK(h, cudaStreamSynchronize(h->stream));
    return MOIL_NB_OK;
}

int moil_nb_set_molecules(moil_nb_ctx *h, const int *mol, const double *mass)
{
    if (!h) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    if (mol && !mass) return MOIL_NB_ERR_ARG;
    cudaSetDevice(h->device);
    if (!h->grp.empty()) {
        for (size_t g = 0; g < h->grp.size(); ++g) {
            const int64_t a0 = h->grp_atom0[g];
            int rc = moil_nb_set_molecules(static_cast<moil_nb_ctx *>(h->grp[g]), mol ? mol + a0 : nullptr,
                                           mol ? mass + a0 : nullptr);
            if (rc != MOIL_NB_OK) { h->err = h->grp[g]->err; return rc; }
        }
        h->nmol = mol ? 1 : 0;
        return MOIL_NB_OK;
    }
    free_ptr(h->d_mol_off); free_ptr(h->d_mol_atom); free_ptr(h->d_mass); free_ptr(h->d_xrel);
    h->nmol = 0;
    if (!mol) return MOIL_NB_OK;
    // CSR over caller atoms: molecules numbered in order of their first atom, atoms ascending
    const size_t n = (size_t)h->natom;
    std::vector<int> off(1, 0), atoms, count;
    std::vector<int> slot(n);
    for (int r = 0; r < h->nrep; ++r) {
        const int a0 = h->rd[r].atom0, na = h->rd[r].natom;
        std::vector<int> id(na, -1);
        for (int a = a0; a < a0 + na; ++a) {
            const int m = mol[a];
            if (m < 0 || m >= na || !(mass[a] >= 0.0) || !std::isfinite(mass[a])) {
                h->err = "molecule index or mass out of range at atom " + std::to_string(a);
                return MOIL_NB_ERR_ARG;
            }
            if (id[m] < 0) { id[m] = (int)count.size(); count.push_back(0); }
            slot[a] = id[m];
            ++count[id[m]];
        }
    }
    const int nmol = (int)count.size();
    off.resize(nmol + 1);
    off[0] = 0;
    for (int m = 0; m < nmol; ++m) off[m + 1] = off[m] + count[m];
    atoms.resize(n);
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (size_t a = 0; a < n; ++a) atoms[fill[slot[a]]++] = (int)a;
    NB_CUDA_OK(h, cudaMalloc(&h->d_mol_off, sizeof(int) * (nmol + 1)));
    NB_CUDA_OK(h, cudaMalloc(&h->d_mol_atom, sizeof(int) * std::max<size_t>(n, 1)));
    NB_CUDA_OK(h, cudaMalloc(&h->d_mass, sizeof(double) * std::max<size_t>(n, 1)));
    NB_CUDA_OK(h, cudaMalloc(&h->d_xrel, sizeof(double) * 3 * std::max<size_t>(n, 1)));
    NB_CUDA_OK(h, cudaMemcpy(h->d_mol_off, off.data(), sizeof(int) * (nmol + 1), cudaMemcpyHostToDevice));
    NB_CUDA_OK(h, cudaMemcpy(h->d_mol_atom, atoms.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    NB_CUDA_OK(h, cudaMemcpy(h->d_mass, mass, sizeof(double) * n, cudaMemcpyHostToDevice));
    h->nmol = nmol;
    return MOIL_NB_OK;
}

int moil_nb_pressure(moil_nb_ctx *h, const double *coor, double *dpot, moil_energies *e, double *press)
{
    if (!h || !coor || !press) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    if (h->nmol == 0) {
        h->err = "no molecules: call moil_nb_set_molecules first";
        return MOIL_NB_ERR_STATE;
    }
    cudaSetDevice(h->device);
    if (!h->grp.empty()) {
        for (size_t g = 0; g < h->grp.size(); ++g) {
            const int64_t a0 = h->grp_atom0[g];
            const int r0 = h->grp_rep0[g];
            int rc = moil_nb_pressure(static_cast<moil_nb_ctx *>(h->grp[g]), coor + 3 * a0,
                                      dpot ? dpot + 3 * a0 : nullptr, e ? e + r0 : nullptr, press + 12 * (size_t)r0);
            if (rc != MOIL_NB_OK) { h->err = h->grp[g]->err; return rc; }
        }
        return MOIL_NB_OK;
    }
    const size_t n = (size_t)h->natom;
    NB_CUDA_OK(h, cudaMemcpyAsync(h->d_coor, coor, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream));
    int rc = eval_impl(h, h->d_coor, h->d_dpot, e);   // lists, positions, PME binning and shares
    if (rc != MOIL_NB_OK) return rc;
    if (!h->d_press_out) {
        NB_CUDA_OK(h, cudaMalloc(&h->d_press_unit, sizeof(double) * 6 * std::max<int64_t>(h->nW + h->nA, 1)));
        NB_CUDA_OK(h, cudaMalloc(&h->d_press_site, sizeof(double) * 3 * std::max<int64_t>(h->nsite, 1)));
        const size_t fp = h->precision == MOIL_NB_FP64 ? sizeof(double) : sizeof(float);
        NB_CUDA_OK(h, cudaMalloc(&h->d_xsite, 4 * fp * std::max<int64_t>(h->nsite, 1)));
        NB_CUDA_OK(h, cudaMalloc(&h->d_press_col, sizeof(double) * 3 * std::max<size_t>(h->cols.size(), 1)));
        NB_CUDA_OK(h, cudaMalloc(&h->d_press_grid, 2 * fp * (h->grid_elems + 2)));
        NB_CUDA_OK(h, cudaMalloc(&h->d_press_out, sizeof(double) * 12 * h->nrep));
    }
    rc = nb_pressure(h, h->d_coor, h->d_press_out);
    if (rc != MOIL_NB_OK) return rc;
    NB_CUDA_OK(h, cudaMemcpyAsync(press, h->d_press_out, sizeof(double) * 12 * h->nrep, cudaMemcpyDeviceToHost,
                                  h->stream));
    if (dpot)
        NB_CUDA_OK(h, cudaMemcpyAsync(dpot, h->d_dpot, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
    NB_CUDA_OK(h, cudaStreamSynchronize(h->stream));
    return MOIL_NB_OK;
}

int moil_nb_get_virial(moil_nb_ctx *h, int replica, double *virvdw)
{
    if (!h || !virvdw) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    if (replica < 0 || replica >= h->nrep) {
        h->err = "replica index out of range";
        return MOIL_NB_ERR_ARG;
    }
    if (!h->grp.empty()) {
        const int g = group_of(h, replica);
        return moil_nb_get_virial(static_cast<moil_nb_ctx *>(h->grp[g]), replica - h->grp_rep0[g], virvdw);
    }
    const double *o = h->h_e_rep + NB_EREP * (size_t)replica;
    for (int k = 0; k < 5; ++k) virvdw[k] = o[12 + k];
    return MOIL_NB_OK;
}

int moil_nb_eval_device(moil_nb_ctx *h, const double *d_coor, double *d_dpot, moil_energies *e)
{
    if (!h || !d_coor || !d_dpot) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    if (!h->grp.empty()) return eval_groups(h, d_coor, d_dpot, e, false);
    return eval_impl(h, d_coor, d_dpot, e);
}

int moil_nb_eval_device_async(moil_nb_ctx *h, const double *d_coor, double *d_dpot)
{
    if (!h || !d_coor || !d_dpot) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    int rc = MOIL_NB_OK;
    if (h->timing) {
        // diagnostic mode runs stage after stage: the whole evaluation here, its status kept
        rc = h->grp.empty() ? eval_impl(h, d_coor, d_dpot, nullptr)
                            : eval_groups(h, d_coor, d_dpot, nullptr, false);
    } else if (!h->grp.empty()) {
        rc = eval_groups(h, d_coor, d_dpot, nullptr, false, 1);
        if (rc != MOIL_NB_OK) return rc;
    } else {
        eval_launch(h, d_coor, d_dpot);
        NB_CUDA_OK(h, cudaPeekAtLastError());
    }
    h->pending = 1;
    h->pend_rc = rc;
    h->pend_coor = d_coor;
    h->pend_dpot = d_dpot;
    return MOIL_NB_OK;
}

int moil_nb_eval_wait(moil_nb_ctx *h, moil_energies *e)
{
    if (!h) return MOIL_NB_ERR_ARG;
    if (!h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    h->pending = 0;
    if (h->timing) {
        if (h->pend_rc == MOIL_NB_OK) {
            if (h->grp.empty()) read_energies(h, e);
            else
                for (size_t g = 0; g < h->grp.size(); ++g) read_energies(h->grp[g], e ? e + h->grp_rep0[g] : nullptr);
        }
        return h->pend_rc;
    }
    if (!h->grp.empty()) return eval_groups(h, h->pend_coor, h->pend_dpot, e, false, 2);
    const int first = eval_complete(h);
    return eval_retry(h, h->pend_coor, h->pend_dpot, e, first, true);
}

int moil_nb_request_rebuild(moil_nb_ctx *h)
{
    if (!h) return MOIL_NB_ERR_ARG;
    if (h->pending) return MOIL_NB_ERR_STATE;
    h->need_rebuild = 1;
    for (NbCtx *c : h->grp) c->need_rebuild = 1;
    return MOIL_NB_OK;
}

int moil_nb_squeeze(const moil_nb_params *p, const moil_topology *t, double *coor)
{
    // symm/squeeze.f:66-145: water and ion monomers move by one box length when their first
    // atom is outside [-L/2, L/2]; y first, then x, then z (the order MOIL tests them)
    if (!p || !t || !coor) return MOIL_NB_ERR_ARG;
    double ha = 0.5 * p->a, hb = 0.5 * p->b, hc = 0.5 * p->c;
    for (int m = 0; m < t->totmon; ++m) {
        if (t->montype[m] == MOIL_MON_OTHER) continue;
        int is = m == 0 ? 0 : t->poipt[m - 1], ie = t->poipt[m];
        double xc = coor[3 * is], yc = coor[3 * is + 1], zc = coor[3 * is + 2];
        for (int k = is; k < ie; ++k) {
            if (yc < -hb) coor[3 * k + 1] += p->b;
            if (yc > hb) coor[3 * k + 1] -= p->b;
            if (xc < -ha) coor[3 * k] += p->a;
            if (zc < -hc) coor[3 * k + 2] += p->c;
            if (xc > ha) coor[3 * k] -= p->a;
            if (zc > hc) coor[3 * k + 2] -= p->c;
        }
    }
    return MOIL_NB_OK;
}

int moil_nb_natoms(const moil_nb_ctx *h, int64_t *n)
{
    if (!h || !n) return MOIL_NB_ERR_ARG;
    *n = h->natom;
    return MOIL_NB_OK;
}

void *moil_nb_stream(const moil_nb_ctx *h) { return h ? (void *)h->stream : nullptr; }

int moil_nb_set_timing(moil_nb_ctx *h, int on)
{
    if (!h) return MOIL_NB_ERR_ARG;
    h->timing = on ? 1 : 0;
    for (NbCtx *c : h->grp) c->timing = h->timing;
    return MOIL_NB_OK;
}

int moil_nb_get_timing(const moil_nb_ctx *h, moil_nb_timing *t)
{
    if (!h || !t) return MOIL_NB_ERR_ARG;
    *t = h->last_timing;
    return MOIL_NB_OK;
}

int moil_nb_pair_stats(const moil_nb_ctx *h, int64_t *list_entries, int64_t *site_pairs)
{
    if (!h) return MOIL_NB_ERR_ARG;
    if (list_entries) *list_entries = h->last_list_entries;
    if (site_pairs) *site_pairs = h->last_site_pairs;
    return MOIL_NB_OK;
}

int moil_nb_set_graph(moil_nb_ctx *h, int on)
{
    if (!h) return MOIL_NB_ERR_ARG;
    cudaSetDevice(h->device);
    h->use_graph = on ? 1 : 0;
    drop_graph(h);
    for (NbCtx *c : h->grp) { c->use_graph = h->use_graph; drop_graph(c); }
    return MOIL_NB_OK;
}

int moil_nb_set_virial(moil_nb_ctx *h, int on)
{
    if (!h) return MOIL_NB_ERR_ARG;
    if (h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    h->virial = on ? 1 : 0;
    drop_graph(h);
    for (NbCtx *c : h->grp) { c->virial = h->virial; drop_graph(c); }
    return MOIL_NB_OK;
}

int moil_nb_set_groups(moil_nb_ctx *h, int groups)
{
    if (!h || groups < 0) return MOIL_NB_ERR_ARG;
    if (h->pending) return MOIL_NB_ERR_STATE;
    h->want_groups = groups;
    return MOIL_NB_OK;
}

int moil_nb_groups(const moil_nb_ctx *h)
{
    return h ? std::max<int>(1, (int)h->grp.size()) : 0;
}

int moil_nb_set_shape(moil_nb_ctx *h, const moil_nb_shape *sp)
{
    if (!h || !sp) return MOIL_NB_ERR_ARG;
    if (h->pending) return MOIL_NB_ERR_STATE;
    if (sp->water_kernel < MOIL_NB_WATER_AUTO || sp->water_kernel > MOIL_NB_WATER_HALF ||
        (sp->half_block != 0 && sp->half_block != 128 && sp->half_block != 256 && sp->half_block != 512) ||
        sp->tiled < MOIL_NB_TILED_AUTO || sp->tiled > MOIL_NB_TILED_ALL || sp->groups < 0) {
        h->err = "moil_nb_set_shape: a field out of range";
        return MOIL_NB_ERR_ARG;
    }
    cudaSetDevice(h->device);
    h->want_groups = sp->groups;
    auto apply = [&](NbCtx *c) -> int {
        c->want_whalf = sp->water_kernel;
        c->hb = sp->half_block ? sp->half_block : 256;
        c->want_tiled = sp->tiled;
        if (!c->inited || !c->grp.empty()) return MOIL_NB_OK;   // a group parent holds no lists
        NB_CUDA_OK(c, cudaStreamSynchronize(c->stream));
        drop_graph(c);
        for (int r = 0; r < c->nrep; ++r) c->rd[r].wtiled = tiled_choice(c, c->rd[r]);
        NB_CUDA_OK(c, cudaMemcpy(c->d_reps, c->rd.data(), sizeof(RepDev) * c->nrep, cudaMemcpyHostToDevice));
        NB_TRY(setup_tiles(c));
        NB_TRY(setup_half(c));
        c->list_gen++;
        c->need_rebuild = 1;
        return MOIL_NB_OK;
    };
    NB_TRY(apply(h));
    for (NbCtx *c : h->grp) {
        const int rc = apply(c);
        if (rc != MOIL_NB_OK) { h->err = c->err; return rc; }
    }
    return MOIL_NB_OK;
}

int moil_nb_get_shape(const moil_nb_ctx *h, moil_nb_shape *sp)
{
    if (!h || !sp) return MOIL_NB_ERR_ARG;
    const NbCtx *c = h->grp.empty() ? h : h->grp[0];
    sp->water_kernel = c->inited ? (c->whalf ? MOIL_NB_WATER_HALF : MOIL_NB_WATER_FULL) : c->want_whalf;
    sp->half_block = c->hb;
    sp->tiled = c->want_tiled;
    sp->groups = h->inited ? moil_nb_groups(h) : h->want_groups;
    return MOIL_NB_OK;
}

// ---- Fortran entry points --------------------------------------------------------
void ewald_init_gpu_(const int *npt, const double *ptchg, const double *epsgm6, const double *epsgm12,
                     const int *exc1, const int *exc2, const int *totspe, const int *spec1, const int *spec2,
                     const double *p14, const int *totmon, const int *poipt, const int *montype,
                     const double *params11, const int *iparams8, int *status)
{
    std::lock_guard<std::mutex> lk(g_fortran_mu);
    if (!status) return;
    if (!npt || !params11 || !iparams8) { *status = MOIL_NB_ERR_ARG; return; }
    if (!g_fortran_ctx) {
        int rc = moil_nb_create(&g_fortran_ctx, 0);
        if (rc != MOIL_NB_OK) { *status = rc; return; }
    }
    moil_nb_params p;
    memset(&p, 0, sizeof p);
    p.rvmx = params11[0]; p.relx = params11[1]; p.eps = params11[2];
    p.a = params11[3]; p.b = params11[4]; p.c = params11[5];
    p.dtol = params11[6]; p.alpha = params11[7]; p.r_on = params11[8]; p.skin = params11[9];
    p.nfft1 = iparams8[0]; p.nfft2 = iparams8[1]; p.nfft3 = iparams8[2]; p.order = iparams8[3];
    p.arith = iparams8[4]; p.hvdw0 = iparams8[5]; p.lj_switch = iparams8[6]; p.precision = iparams8[7];
    p.list_period = (int)params11[10];
    moil_topology t;
    t.npt = *npt; t.ptchg = ptchg; t.epsgm6 = epsgm6; t.epsgm12 = epsgm12; t.exc1 = exc1; t.exc2 = exc2;
    t.totspe = totspe ? *totspe : 0; t.spec1 = spec1; t.spec2 = spec2; t.p14 = p14;
    t.totmon = totmon ? *totmon : 0; t.poipt = poipt; t.montype = montype;
    *status = moil_nb_init(g_fortran_ctx, &p, &t);
}

void nblist_gpu_(int *status)
{
    std::lock_guard<std::mutex> lk(g_fortran_mu);
    if (!status) return;
    *status = g_fortran_ctx ? moil_nb_request_rebuild(g_fortran_ctx) : MOIL_NB_ERR_STATE;
}

void eforce_nb_gpu_(const int *npt, const double *coor, double *dpot, double *enb, int *status)
{
    // MOIL's terms accumulate into dpot (pot/eforce.f:64-68 zeroes it first), so this entry
    // adds the nonbonded gradient to what the caller already holds.
    std::lock_guard<std::mutex> lk(g_fortran_mu);
    if (!status) return;
    if (!g_fortran_ctx || !npt || !coor || !dpot) { *status = g_fortran_ctx ? MOIL_NB_ERR_ARG : MOIL_NB_ERR_STATE; return; }
    if ((int64_t)*npt != g_fortran_ctx->natom) { *status = MOIL_NB_ERR_ARG; return; }
    g_fortran_buf.resize(3 * (size_t)*npt);
    moil_energies e;
    int rc = moil_nb_eval(g_fortran_ctx, coor, g_fortran_buf.data(), &e);
    if (rc == MOIL_NB_OK) {
        for (size_t k = 0; k < g_fortran_buf.size(); ++k) dpot[k] += g_fortran_buf[k];
        if (enb) {
            const double v[11] = {e.e_vdw, e.e_el, e.e_vsym, e.e_lsym, e.e_el14, e.e_vdw14,
                                  e.e_corr, e.e_self, e.e_ew_receip, e.e_total, e.e_dir};
            memcpy(enb, v, sizeof v);
        }
    }
    *status = rc;
}

void eforce_nb_press_gpu_(const int *npt, const double *coor, double *dpot, double *enb, double *virvdw,
                          int *status)
{
    {
        std::lock_guard<std::mutex> lk(g_fortran_mu);
        if (g_fortran_ctx && !g_fortran_ctx->virial) moil_nb_set_virial(g_fortran_ctx, 1);
    }
    eforce_nb_gpu_(npt, coor, dpot, enb, status);
    if (!status || *status != MOIL_NB_OK || !virvdw) return;
    std::lock_guard<std::mutex> lk(g_fortran_mu);
    *status = moil_nb_get_virial(g_fortran_ctx, 0, virvdw);
}

}  // extern "C"

// ---- device-side MD step loop (moil_nb_md_step) -----------------------------------------
void read_energies_of(NbCtx *c, moil_energies *e) { read_energies(c, e); }

int nb_md_loop(NbCtx *c, double *coor, double *vel, const double *mass, double *dpot, double dt, double doh,
               double dhh, int nsteps)
{
    cudaStream_t s = c->stream;
    if (!c->d_mdctl) NB_CUDA_OK(c, cudaMalloc(&c->d_mdctl, sizeof(int) * 4));
    // the host's list schedule goes to the device once per call
    c->h_status[17] = c->evals_since_build;
    c->h_status[18] = c->need_rebuild ? 1 : 0;
    c->h_status[19] = 0;
    NB_CUDA_OK(c, cudaMemcpyAsync(c->d_mdctl, c->h_status + 17, sizeof(int) * 3, cudaMemcpyHostToDevice, s));
    const bool same = c->gexec_md && c->gmd_key[0] == coor && c->gmd_key[1] == vel && c->gmd_key[2] == mass &&
                      c->gmd_dt == dt && c->gmd_doh == doh && c->gmd_dhh == dhh && c->gmd_gen == c->list_gen &&
                      c->gmd_dpot == dpot;
    if (!same) {
        if (c->gexec_md) cudaGraphExecDestroy(c->gexec_md);
        c->gexec_md = nullptr;
        cudaGraph_t g = nullptr;
        NB_CUDA_OK(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        c->capturing = 1;
        const bool built = enqueue_md_step(c, coor, vel, mass, dpot, dt, doh, dhh);
        c->capturing = 0;
        cudaError_t e1 = cudaStreamEndCapture(s, &g);
        cudaError_t e2 = e1 == cudaSuccess ? (built ? cudaGraphInstantiate(&c->gexec_md, g, 0) : cudaErrorNotSupported) : e1;
        if (g) cudaGraphDestroy(g);
        if (e2 != cudaSuccess) {
            c->gexec_md = nullptr;
            c->err = std::string("capturing the MD step graph: ") + cudaGetErrorString(e2);
            return MOIL_NB_ERR_CUDA;
        }
        c->gmd_key[0] = coor; c->gmd_key[1] = vel; c->gmd_key[2] = mass;
        c->gmd_dpot = dpot;
        c->gmd_dt = dt; c->gmd_doh = doh; c->gmd_dhh = dhh;
        c->gmd_gen = c->list_gen;
    }
    for (int k = 0; k < nsteps; ++k) NB_CUDA_OK(c, cudaGraphLaunch(c->gexec_md, s));
    // the last step's status words and energies, and the step control, in one wait
    NB_CUDA_OK(c, cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int) * 8, cudaMemcpyDeviceToHost, s));
    NB_CUDA_OK(c, cudaMemcpyAsync(c->h_e_rep, c->d_e_rep, sizeof(double) * NB_EREP * c->nrep,
                                  cudaMemcpyDeviceToHost, s));
    NB_CUDA_OK(c, cudaMemcpyAsync(c->h_status + 20, c->d_mdctl, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
    return MOIL_NB_OK;
}
