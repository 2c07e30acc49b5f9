// nb_lists.cu -- list rebuild: the GPU replacement of squeeze()/nbondm()/nbond()/syminit().
//
// MOIL builds an O(M^2) monomer list (pot/nbondm.f:143-210), atom lists with exclusion and
// hydrogen filters (pot/nbond.f:54-157) and 13 image-translation lists (symm/nbmsym.f,
// symm/nbsym.f).  Here the same pair set comes from a cell list with minimum-image
// distances (identical for cutoff <= L/2):
//   units     : water molecules (anchor O, pot/nbondm.f:81-86) and non-water atoms
//   sort      : counting sort of units by (class, replica, cell), ties by unit id
//   lists     : W1  water i -> water j   (O-O < rmax + skin)      fixed-capacity rows
//               W2  water i -> non-water site j (O-x < rmax + skin + rwat)     CSR
//               X   non-water i -> any site j (exclusions removed, as pot/nbond.f:95-103)  CSR
// Every list is full (both directions) so each lane owns its gradient outright.
// All kernels that only run on a rebuild early-exit on the device rebuild flag, so the
// whole evaluation can run without a host round trip.
#include "nb_internal.h"

namespace {

__device__ __forceinline__ bool rebuild_off(const int *st) { return st[0] == 0; }

// ---------------------------------------------------------------------------------
// 1. unit -> cell key (anchor wrapped into [0, L)), histogram slot
__global__ void k_unit_keys(int nunit, int nW, int ncell, const int *__restrict__ unit_atom,
                            const int *__restrict__ unit_rep, const RepDev *__restrict__ reps,
                            const double *__restrict__ coor, int *__restrict__ key, int *__restrict__ slot,
                            int *__restrict__ hist, int *st)
{
    if (rebuild_off(st)) return;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nunit; u += gridDim.x * blockDim.x) {
        const RepDev &R = reps[unit_rep[u]];
        int a = unit_atom[u];
        int ci[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double x = coor[3 * (size_t)a + d];
            if (!(x == x) || fabs(x) > 1e7) { atomicOr(&st[1], NB_DEV_ERR_NAN); x = 0.0; }
            double f = x * R.invLd[d] + 0.5;
            f -= floor(f);
            int q = (int)(f * R.nc[d]);
            ci[d] = q >= R.nc[d] ? R.nc[d] - 1 : (q < 0 ? 0 : q);
        }
        int cell = R.cell0 + ci[0] + R.nc[0] * (ci[1] + R.nc[1] * ci[2]);
        int k = (u < nW ? 0 : ncell) + cell;
        key[u] = k;
        slot[u] = atomicAdd(&hist[k], 1);
    }
}

__global__ void k_unit_scatter(int nunit, const int *__restrict__ key, const int *__restrict__ slot,
                               const int *__restrict__ start, int *__restrict__ sorted, const int *st)
{
    if (rebuild_off(st)) return;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nunit; u += gridDim.x * blockDim.x)
        sorted[start[key[u]] + slot[u]] = u;
}

// deterministic order inside a bin: ascending unit id.  One warp per bin: the bin is staged
// in shared memory and each unit goes to its rank (ids are distinct); bins longer than the
// stage fall back to an insertion sort by one lane.
#define NB_BIN_STAGE 1024
__global__ void __launch_bounds__(128) k_bin_sort(int nbin, const int *__restrict__ start, int *__restrict__ sorted,
                                                  const int *st)
{
    if (rebuild_off(st)) return;
    __shared__ int stage[4][NB_BIN_STAGE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *v = stage[warp];
    for (int b = blockIdx.x * 4 + warp; b < nbin; b += gridDim.x * 4) {
        const int lo = start[b], n = start[b + 1] - lo;
        if (n <= 1) continue;
        if (n > NB_BIN_STAGE) {
            if (lane == 0)
                for (int i = lo + 1; i < lo + n; ++i) {
                    int x = sorted[i], j = i - 1;
                    while (j >= lo && sorted[j] > x) { sorted[j + 1] = sorted[j]; --j; }
                    sorted[j + 1] = x;
                }
            __syncwarp();
            continue;
        }
        for (int k = lane; k < n; k += 32) v[k] = sorted[lo + k];
        __syncwarp();
        for (int k = lane; k < n; k += 32) {
            const int x = v[k];
            int r = 0;
            for (int m = 0; m < n; ++m) r += v[m] < x;
            sorted[lo + r] = x;
        }
        __syncwarp();
    }
}

// 2. sites from the sorted units
template <typename T>
__global__ void k_site_build(int nunit, int nW, const int *__restrict__ sorted, const int *__restrict__ unit_atom,
                             const int *__restrict__ atom_rep, const unsigned *__restrict__ aflags,
                             const float2 *__restrict__ lj_f, const double2 *__restrict__ lj_d,
                             const double *__restrict__ q, int *__restrict__ site_orig, int *__restrict__ site_of,
                             int *__restrict__ site_rep, unsigned *__restrict__ site_flags, void *site_lj_v,
                             void *site_q_v, const int *st)
{
    if (rebuild_off(st)) return;
    typedef typename cplx<T>::type T2;
    T2 *site_lj = (T2 *)site_lj_v;
    T *site_q = (T *)site_q_v;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nunit; p += gridDim.x * blockDim.x) {
        int u = sorted[p];
        int a0 = unit_atom[u];
        int s0, ns;
        if (p < nW) { s0 = 3 * p; ns = 3; } else { s0 = 3 * nW + (p - nW); ns = 1; }
        for (int k = 0; k < ns; ++k) {
            int a = a0 + k, s = s0 + k;
            site_orig[s] = a;
            site_of[a] = s;
            site_rep[s] = atom_rep[a];
            site_flags[s] = aflags[a];
            if (sizeof(T) == 4) {
                float2 v = lj_f[a];
                ((float2 *)site_lj)[s] = v;
            } else {
                double2 v = lj_d[a];
                ((double2 *)site_lj)[s] = v;
            }
            site_q[s] = (T)q[a];
        }
    }
}

// 3. per-evaluation coordinate conversion into site order; displacement check.  One thread
// per sorted water (its three consecutive caller atoms, 72 contiguous bytes) or non-water
// site, so every site-order array is read and written coalesced.
// Sites that do not track (water hydrogens) neither read nor write their build position.
template <typename T>
__device__ __forceinline__ void prepare_site(int s, const double *x, const unsigned *__restrict__ site_flags,
                                             const T *__restrict__ site_q, void *pos_v, float4 *__restrict__ posb,
                                             float half_skin2, int snapshot, bool track, bool &moved)
{
    typedef typename vec4<T>::type T4;
    const unsigned f = site_flags[s];
    T4 p;
    p.x = (T)x[0]; p.y = (T)x[1]; p.z = (T)x[2];
    p.w = (f & SF_CHARGED) ? site_q[s] : (T)0;
    ((T4 *)pos_v)[s] = p;
    if (!track) return;
    const float4 pf = make_float4((float)x[0], (float)x[1], (float)x[2], 0.f);
    if (snapshot) {
        posb[s] = pf;
    } else {
        // lists stay valid while no site moved more than skin/2 since the build
        const float4 b = posb[s];
        const float dx = pf.x - b.x, dy = pf.y - b.y, dz = pf.z - b.z;
        moved |= dx * dx + dy * dy + dz * dz > half_skin2;
    }
}

// coordinates of one caller atom; a non-finite or absurd one (|x| > 1e7, NaN, inf) is
// reported and replaced by 0.  The test runs on the bit pattern: |x| > 1e7 exactly when the
// magnitude bits exceed those of 1e7 (0x416312D000000000), NaN and inf included, and costs
// no FP64 instruction (the FP64 pipe is a small fraction of the FP32 one)
__device__ __forceinline__ void load_atom(const double *__restrict__ coor, int a, double *x, int *st)
{
    x[0] = coor[3 * (size_t)a]; x[1] = coor[3 * (size_t)a + 1]; x[2] = coor[3 * (size_t)a + 2];
    const unsigned long long m = 0x7fffffffffffffffULL, lim = 0x416312D000000000ULL;
    if (((unsigned long long)__double_as_longlong(x[0]) & m) > lim ||
        ((unsigned long long)__double_as_longlong(x[1]) & m) > lim ||
        ((unsigned long long)__double_as_longlong(x[2]) & m) > lim) {
        atomicOr(&st[1], NB_DEV_ERR_NAN);
        x[0] = x[1] = x[2] = 0.0;
    }
}

template <typename T>
__global__ void k_prepare(int nW, int nA, const int *__restrict__ site_orig, const unsigned *__restrict__ site_flags,
                          const void *site_q_v, const double *__restrict__ coor, void *pos_v, void *woff_v,
                          float4 *__restrict__ posb, float half_skin2, float rwat2, int snapshot, int *st)
{
    // snapshot mode runs only on a rebuild; check mode only without one (the site order it
    // reads is the previous build's, which does not exist before the first build)
    if (snapshot ? rebuild_off(st) : !rebuild_off(st)) return;
    typedef typename vec4<T>::type T4;
    const T *site_q = (const T *)site_q_v;
    bool moved = false;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nW + nA; u += gridDim.x * blockDim.x) {
        if (u < nW) {
            // a water's caller atoms are consecutive (O, H, H), as are its sites
            const int a = site_orig[3 * u];
            double x[3][3];
#pragma unroll
            for (int m = 0; m < 3; ++m) load_atom(coor, a + m, x[m], st);
            // only the oxygen's displacement counts: every water list is built from oxygen
            // distances with radii that include the hydrogens' reach (rwat, checked below)
#pragma unroll
            for (int m = 0; m < 3; ++m)
                prepare_site<T>(3 * u + m, x[m], site_flags, site_q, pos_v, posb, half_skin2, snapshot, m == 0,
                                moved);
            // the molecule record of the water kernel: O position (and charge), then the offsets
            ((T4 *)woff_v)[3 * u] = ((const T4 *)pos_v)[3 * u];
#pragma unroll
            for (int m = 1; m < 3; ++m) {
                // H offset from its O, formed in FP64 so the water kernel's site displacements
                // inherit no extra rounding from absolute FP32 positions; water sites must stay
                // within rwat of their oxygen (list radius assumption)
                T4 off;
                off.x = (T)(x[m][0] - x[0][0]); off.y = (T)(x[m][1] - x[0][1]); off.z = (T)(x[m][2] - x[0][2]);
                off.w = (T)0;
                if (off.x * off.x + off.y * off.y + off.z * off.z > (T)rwat2) atomicOr(&st[1], NB_DEV_ERR_RWAT);
                ((T4 *)woff_v)[3 * u + m] = off;
            }
        } else {
            const int s = 3 * nW + (u - nW);
            double x[3];
            load_atom(coor, site_orig[s], x, st);
            prepare_site<T>(s, x, site_flags, site_q, pos_v, posb, half_skin2, snapshot, true, moved);
        }
    }
    if (moved) atomicOr(&st[0], 1);
}

// unique neighbour cells along one axis
__device__ __forceinline__ int nb_axis_cells(int c, int n, int out[3])
{
    int m = 0;
    for (int t = -1; t <= 1; ++t) {
        int v = c + t;
        v = v < 0 ? v + n : (v >= n ? v - n : v);
        bool dup = false;
        for (int k = 0; k < m; ++k) dup |= (out[k] == v);
        if (!dup) out[m++] = v;
    }
    return m;
}

template <typename T>
__device__ __forceinline__ void cell_of(const RepDev &R, T x, T y, T z, int ci[3])
{
    T p[3] = {x, y, z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        T f = p[d] * rep_invL<T>(R, d) + (T)0.5;
        f -= floor(f);
        int q = (int)(f * R.nc[d]);
        ci[d] = q >= R.nc[d] ? R.nc[d] - 1 : (q < 0 ? 0 : q);
    }
}

template <typename T>
__device__ __forceinline__ T mi_r2(const RepDev &R, T dx, T dy, T dz)
{
    dx -= rep_L<T>(R, 0) * nb_rint(dx * rep_invL<T>(R, 0));
    dy -= rep_L<T>(R, 1) * nb_rint(dy * rep_invL<T>(R, 1));
    dz -= rep_L<T>(R, 2) * nb_rint(dz * rep_invL<T>(R, 2));
    return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ bool nb_excluded(const int *__restrict__ ex_off, const int *__restrict__ ex_j, int a, int b)
{
    for (int k = ex_off[a]; k < ex_off[a + 1]; ++k)
        if (ex_j[k] == b) return true;
    return false;
}

// W1 is a fixed-capacity row per water (ELL, cap entries): molecules inside the cutoff at
// build time from the front of the row in ascending order of discovery, skin-only
// molecules from the back, counts (near, far) in wcnt[i].  The pair kernel walks the front
// part then the back part, so the lanes of a warp stay converged over the in-cutoff part.
// E: the row entry type, int32 sorted water indices or (every replica below 65,536 waters)
// uint16 indices relative to the replica's first water, which halves the row stream the
// water kernel reads every evaluation
template <typename E>
__device__ __forceinline__ void w1_put(E *__restrict__ row, int cap, bool near, int &nn, int &nf, int j)
{
    if (near) { if (nn < cap) row[nn] = (E)j; ++nn; }
    else { if (nf < cap) row[cap - 1 - nf] = (E)j; ++nf; }
}
template <typename E> __device__ __forceinline__ int row_base(const RepDev &R) { return sizeof(E) == 2 ? R.wat0 : 0; }

// a finished W1 row: counts, overflow flag, and the warp's entry total / longest row added
// to st[2] / st[6] (for statistics and for regrowing the row capacity)
__device__ __forceinline__ void w1_done(int i, int nn, int nf, int cap, int2 *__restrict__ wcnt, int *st)
{
    wcnt[i] = make_int2(nn, nf);
    const int n = nn + nf;
    if (n > cap) atomicOr(&st[1], NB_DEV_ERR_OVERFLOW);
    const unsigned act = __activemask();
    const int sum = __reduce_add_sync(act, n), mx = __reduce_max_sync(act, n);
    if ((threadIdx.x & 31) == __ffs(act) - 1) {
        atomicAdd(&st[2], sum);
        atomicMax(&st[6], mx);
    }
}

// 4. water lists of water i by cell search: W1 (water j, rows of wl1) in the FILL = 0 pass,
// W2 (non-water sites, CSR) counted in the FILL = 0 pass and written in the FILL = 1 pass
template <typename T, int FILL, typename E>
__device__ __forceinline__ void wlist_one(int i, int nW, const RepDev *__restrict__ reps,
                                          const int *__restrict__ site_rep, const void *pos_v,
                                          const int *__restrict__ bin_start, int ncell, int2 *__restrict__ wcnt,
                                          int *__restrict__ cnt2, const int *__restrict__ off2, void *__restrict__ l1,
                                          int cap_row, int *__restrict__ l2, int64_t cap2, int *st)
{
    typedef typename vec4<T>::type T4;
    const T4 *pos = (const T4 *)pos_v;
    const RepDev &R = reps[site_rep[3 * i]];
    const bool do_w1 = !FILL && !R.wtiled;   // replicas with few cells: W1 from k_wlist_tiled
    if (!do_w1 && R.noth == 0) {
        if (!FILL) cnt2[i] = 0;
        return;
    }
    T4 oi = pos[3 * i];
    int ci[3], cx[3], cy[3], cz[3];
    cell_of<T>(R, oi.x, oi.y, oi.z, ci);
    int nx = nb_axis_cells(ci[0], R.nc[0], cx), ny = nb_axis_cells(ci[1], R.nc[1], cy),
        nz = nb_axis_cells(ci[2], R.nc[2], cz);
    int n2 = 0, nn = 0, nf = 0;
    int w2 = FILL ? off2[i] : 0;
    E *row = (E *)l1 + (size_t)i * cap_row;
    T rl2 = (T)R.rlist2, rw2 = (T)R.rlistw2, rc2 = (T)R.rmax2;
    int nW_i = nW;
    for (int a = 0; a < nz; ++a)
        for (int b = 0; b < ny; ++b)
            for (int d = 0; d < nx; ++d) {
                int cell = R.cell0 + cx[d] + R.nc[0] * (cy[b] + R.nc[1] * cz[a]);
                // waters in the cell: sorted positions [bin_start[cell], bin_start[cell+1])
                if (do_w1)
                    for (int p = bin_start[cell]; p < bin_start[cell + 1]; ++p) {
                        if (p == i) continue;
                        T4 oj = pos[3 * p];
                        T r2 = mi_r2<T>(R, oi.x - oj.x, oi.y - oj.y, oi.z - oj.z);
                        if (r2 < rl2) w1_put(row, cap_row, r2 <= rc2, nn, nf, p - row_base<E>(R));
                    }
                // non-water atoms in the cell
                for (int p = bin_start[ncell + cell]; p < bin_start[ncell + cell + 1]; ++p) {
                    int s = 3 * nW_i + (p - nW_i);
                    T4 xj = pos[s];
                    if (mi_r2<T>(R, oi.x - xj.x, oi.y - xj.y, oi.z - xj.z) < rw2) {
                        if (FILL) { if (w2 + n2 < cap2) l2[w2 + n2] = s; }
                        n2++;
                    }
                }
            }
    if (!FILL) {
        cnt2[i] = n2;
        if (do_w1) w1_done(i, nn, nf, cap_row, wcnt, st);
    }
    else if ((int64_t)w2 + n2 > cap2) atomicOr(&st[1], NB_DEV_ERR_OVERFLOW);
}

template <typename T, int FILL, typename E>
__global__ void k_wlist(int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep, const void *pos_v,
                        const int *__restrict__ bin_start, int ncell, int2 *__restrict__ wcnt,
                        int *__restrict__ cnt2, const int *__restrict__ off2, void *__restrict__ l1, int cap_row,
                        int *__restrict__ l2, int64_t cap2, int *st)
{
    if (rebuild_off(st)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nW; i += gridDim.x * blockDim.x)
        wlist_one<T, FILL, E>(i, nW, reps, site_rep, pos_v, bin_start, ncell, wcnt, cnt2, off2, l1, cap_row, l2, cap2,
                           st);
}

// oxygen position wrapped into [0, L) per axis, as FP32 (list geometry only)
template <typename T>
__device__ __forceinline__ float4 wrap_box(const RepDev &R, typename vec4<T>::type p)
{
    T x = p.x - rep_L<T>(R, 0) * floor(p.x * rep_invL<T>(R, 0));
    T y = p.y - rep_L<T>(R, 1) * floor(p.y * rep_invL<T>(R, 1));
    T z = p.z - rep_L<T>(R, 2) * floor(p.z * rep_invL<T>(R, 2));
    return make_float4((float)x, (float)y, (float)z, 0.f);
}

// 4b. W1 for replicas whose cell stencil spans most of the box (k_wlist_tiled): all
// molecule pairs of the replica in one pass, oxygens staged in shared-memory tiles of
// NB_WTILE (x, y and z arrays) and read by broadcast, two molecules per packed FP32x2
// operation.  One block = NB_WTILE consecutive sorted waters of one replica (blocks never
// straddle replicas).  Each 32-molecule word of a tile gives a bit set (within the list
// radius) and a near set (within the cutoff) whose members go to the row in ascending j.
__device__ __forceinline__ float2 pf2(float a) { return make_float2(a, a); }

// bounding boxes: each warp's i molecules and each 32-molecule word of a tile (positions
// wrapped into [0, L)); a word whose box is farther than the list radius from the warp's box
// in every image is skipped by the whole warp
__device__ __forceinline__ void warp_box(bool valid, float x, float y, float z, float lo[3], float hi[3])
{
    lo[0] = valid ? x : 3.0e38f; lo[1] = valid ? y : 3.0e38f; lo[2] = valid ? z : 3.0e38f;
    hi[0] = valid ? x : -3.0e38f; hi[1] = valid ? y : -3.0e38f; hi[2] = valid ? z : -3.0e38f;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
}

template <typename T, typename E>
__device__ __forceinline__ void wlist_tile(int2 w, float (*sj)[NB_WTILE], float (*sbb)[6],
                                           const RepDev *__restrict__ reps, const void *pos_v,
                                           int2 *__restrict__ wcnt, void *__restrict__ l1, int cap_row, int *st)
{
    typedef typename vec4<T>::type T4;
    const T4 *pos = (const T4 *)pos_v;
    const RepDev &R = reps[w.x];
    const int j0 = R.wat0, nw = R.nwat;
    const int i = w.y + (int)threadIdx.x, il = i - j0;
    const bool act = il < nw;
    const float rl2 = R.rlist2, rc2 = R.rmax2;
    const float4 oi = act ? wrap_box<T>(R, pos[3 * (size_t)i]) : make_float4(0.f, 0.f, 0.f, 0.f);
    // minimum image of positions wrapped into [0, L): d - L rint(d / L), the rounding by the
    // 1.5 * 2^23 shift (|d / L| < 1)
    const float2 o[3] = {pf2(oi.x), pf2(oi.y), pf2(oi.z)};
    const float2 iL[3] = {pf2(R.invL[0]), pf2(R.invL[1]), pf2(R.invL[2])};
    const float2 nL[3] = {pf2(-R.L[0]), pf2(-R.L[1]), pf2(-R.L[2])};
    const float2 mg = pf2(12582912.f), nmg = pf2(-12582912.f), m1 = pf2(-1.f);
    const float2 nrl2 = pf2(-rl2), nrc2 = pf2(-rc2);
    E *row = (E *)l1 + (size_t)i * cap_row;
    int nn = 0, nf = 0;
    float ilo[3], ihi[3];
    warp_box(act, oi.x, oi.y, oi.z, ilo, ihi);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t0 = 0; t0 < nw; t0 += NB_WTILE) {
        __syncthreads();
        const bool has = t0 + (int)threadIdx.x < nw;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        if (has) {
            p = wrap_box<T>(R, pos[3 * (size_t)(j0 + t0 + threadIdx.x)]);
            sj[0][threadIdx.x] = p.x;
            sj[1][threadIdx.x] = p.y;
            sj[2][threadIdx.x] = p.z;
        }
        {
            // the box of the word this warp loaded
            float lo[3], hi[3];
            warp_box(has, p.x, p.y, p.z, lo, hi);
            if (lane == 0)
                for (int d = 0; d < 3; ++d) { sbb[warp][d] = lo[d]; sbb[warp][3 + d] = hi[d]; }
        }
        __syncthreads();
        if (!act) continue;
        const int tn = min(NB_WTILE, nw - t0);
#pragma unroll
        for (int q = 0; q < NB_WTILE / 32; ++q) {
            const int nv = tn - 32 * q;
            if (nv <= 0) break;
            {
                // separation of the boxes over the images (-L, 0, +L) per axis
                float s2 = 0.f;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float jlo = sbb[q][d], jhi = sbb[q][3 + d], L = R.L[d];
                    const float s0 = fmaxf(0.f, fmaxf(jlo - ihi[d], ilo[d] - jhi));
                    const float sp = fmaxf(0.f, jlo + L - ihi[d]), sm = fmaxf(0.f, ilo[d] - jhi + L);
                    const float sd = fminf(s0, fminf(sp, sm));
                    s2 = fmaf(sd, sd, s2);
                }
                if (s2 >= rl2) continue;
            }
            unsigned m = 0u, mn = 0u;
#pragma unroll 4
            for (int b = 0; b < 32; b += 2) {
                float2 r2 = pf2(0.f);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float2 p = *reinterpret_cast<const float2 *>(&sj[d][32 * q + b]);
                    float2 x = __ffma2_rn(p, m1, o[d]);                               // o - p
                    const float2 n = __fadd2_rn(__ffma2_rn(x, iL[d], mg), nmg);
                    x = __ffma2_rn(n, nL[d], x);
                    r2 = __ffma2_rn(x, x, r2);
                }
                // r2 < r as the sign bit of r2 - r, one packed subtraction for both molecules
                const float2 dl = __fadd2_rn(r2, nrl2), dc = __fadd2_rn(r2, nrc2);
                m |= ((__float_as_uint(dl.x) >> 31) | ((__float_as_uint(dl.y) >> 31) << 1)) << b;
                mn |= ((__float_as_uint(dc.x) >> 31) | ((__float_as_uint(dc.y) >> 31) << 1)) << b;
            }
            unsigned keep = nv < 32 ? (1u << nv) - 1u : 0xffffffffu;   // past the last molecule
            const int self = il - t0 - 32 * q;
            if ((unsigned)self < 32u) keep &= ~(1u << self);
            m &= keep;
            mn &= m;
            const int jb = j0 + t0 + 32 * q;
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1u;
                w1_put(row, cap_row, (mn >> b) & 1u, nn, nf, jb + b - row_base<E>(R));
            }
        }
    }
    if (act) w1_done(i, nn, nf, cap_row, wcnt, st);
}

template <typename T, typename E>
__global__ void __launch_bounds__(NB_WTILE) k_wlist_tiled(int ntile, const int2 *__restrict__ work,
                                                          const RepDev *__restrict__ reps, const void *pos_v,
                                                          int2 *__restrict__ wcnt, void *__restrict__ l1, int cap_row,
                                                          int *st)
{
    if (rebuild_off(st)) return;
    __shared__ __align__(16) float sj[3][NB_WTILE];
    __shared__ float sbb[NB_WTILE / 32][6];
    // every tile pass starts with a block barrier before it overwrites sj and sbb
    for (int b = blockIdx.x; b < ntile; b += gridDim.x)
        wlist_tile<T, E>(work[b], sj, sbb, reps, pos_v, wcnt, l1, cap_row, st);
}

// 4c. Half water rows for the FP32 half-list water kernel (k_water_h).  Every water-water
// pair of the full W1 rows is kept once, under its owner (nb_half_owner: an index-parity
// rule that gives every water about half of its partners, so lanes stay balanced).  One
// block = HB consecutive sorted waters of one replica (the k_water_h block); its j-set is
// the sorted set of partners its rows own, found with a bitmap over the replica's waters
// and a block scan of the word popcounts.  Row entry k of lane t sits at k * HB + t (the
// kernel's loads coalesce) and packs (j-set index << 16) | (j's offset from the replica's
// first water); owned in-cutoff partners first, as in the full row.  The block's longest
// row and its j-set size go to st[7] and st[5] (capacity regrowth).
#define NB_HB_WORDS 2048     // bitmap words: replicas of up to 65,536 waters (16-bit rows)
template <int HB>
__global__ void __launch_bounds__(HB) k_whalf(int nblk, const int2 *__restrict__ blocks,
                                              const RepDev *__restrict__ reps, const int2 *__restrict__ wcnt,
                                              const unsigned short *__restrict__ wl1, int cap_row,
                                              unsigned *__restrict__ hrow, int caph, int2 *__restrict__ hcnt,
                                              int *__restrict__ jset, int *__restrict__ jn, int jcap, int *st)
{
    if (rebuild_off(st)) return;
    __shared__ unsigned bits[NB_HB_WORDS];
    __shared__ int pre[NB_HB_WORDS];
    __shared__ int wsum[HB / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int b = blockIdx.x; b < nblk; b += gridDim.x) {
        const int2 w = blocks[b];
        const RepDev &R = reps[w.x];
        const int nwords = (R.nwat + 31) >> 5;
        __syncthreads();    // the previous block's bitmap and prefix are no longer read
        for (int k = t; k < nwords; k += HB) bits[k] = 0u;
        __syncthreads();
        const int i = w.y + t, il = i - R.wat0;
        const bool act = il < R.nwat;
        const int2 c = act ? wcnt[i] : make_int2(0, 0);
        // an overflowed row is read within its capacity (the evaluation is redone)
        const int nn = min(c.x, cap_row), nf = min(c.x + c.y, cap_row) - nn;
        const unsigned short *row = wl1 + (size_t)i * cap_row;
        // the row's entries, eight at a time (16-byte loads; rows start 64-byte aligned): the
        // in-cutoff ones [0, nn), then the skin ones [cap_row - nf, cap_row)
        auto for_row = [&](auto fn) {
            for (int v0 = 0; v0 < nn; v0 += 8) {
                const uint4 q = *reinterpret_cast<const uint4 *>(row + v0);
                const unsigned u[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    if (v0 + e < nn) fn((int)((u[e >> 1] >> (16 * (e & 1))) & 0xffffu), true);
            }
            for (int v0 = (cap_row - nf) & ~7; v0 < cap_row; v0 += 8) {
                const uint4 q = *reinterpret_cast<const uint4 *>(row + v0);
                const unsigned u[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    if (v0 + e >= cap_row - nf) fn((int)((u[e >> 1] >> (16 * (e & 1))) & 0xffffu), false);
            }
        };
        for_row([&](int jl, bool) {
            if (nb_half_owner(il, jl) == il) atomicOr(&bits[jl >> 5], 1u << (jl & 31));
        });
        __syncthreads();
        // exclusive prefix of the word popcounts: each thread a contiguous chunk of words
        const int per = (nwords + HB - 1) / HB, k0 = min(t * per, nwords), k1 = min(k0 + per, nwords);
        int s = 0;
        for (int k = k0; k < k1; ++k) s += __popc(bits[k]);
        int x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        int base = 0, total = 0;
#pragma unroll
        for (int q = 0; q < HB / 32; ++q) {
            base += q < warp ? wsum[q] : 0;
            total += wsum[q];
        }
        int run = base + x - s;
        for (int k = k0; k < k1; ++k) {
            pre[k] = run;
            run += __popc(bits[k]);
        }
        __syncthreads();
        // the j-set in ascending water order
        for (int k = t; k < nwords; k += HB) {
            unsigned m = bits[k];
            int p = pre[k];
            while (m) {
                const int bb = __ffs(m) - 1;
                m &= m - 1u;
                if (p < jcap) jset[(size_t)b * jcap + p] = R.wat0 + 32 * k + bb;
                ++p;
            }
        }
        // the owned entries, in the full row's order (in-cutoff partners first)
        unsigned *hr = hrow + (size_t)b * caph * HB + t;
        int kin = 0, kt = 0;
        for_row([&](int jl, bool near) {
            if (nb_half_owner(il, jl) != il) return;
            const int loc = pre[jl >> 5] + __popc(bits[jl >> 5] & ((1u << (jl & 31)) - 1u));
            if (kt < caph) hr[(size_t)kt * HB] = ((unsigned)loc << 16) | (unsigned)jl;
            ++kt;
            kin += near;
        });
        // a j-set beyond its capacity leaves the block's rows empty (the evaluation is redone
        // with a larger one), so no entry indexes past the kernel's accumulators
        if (act) hcnt[i] = total > jcap ? make_int2(0, 0) : make_int2(min(kin, caph), min(kt, caph));
        const int mx = __reduce_max_sync(0xffffffffu, kt);
        if (lane == 0) atomicMax(&st[7], mx);
        if (t == 0) {
            jn[b] = min(total, jcap);
            atomicMax(&st[5], total);
        }
        if (kt > caph || (t == 0 && total > jcap)) atomicOr(&st[1], NB_DEV_ERR_OVERFLOW);
    }
}

// 5. non-water list X: every site j within reach, exclusions removed
template <typename T, int FILL>
__device__ __forceinline__ void xlist_one(int k, int nW, const RepDev *__restrict__ reps,
                                          const int *__restrict__ site_rep, const int *__restrict__ site_orig,
                                          const void *pos_v, const int *__restrict__ bin_start, int ncell,
                                          const int *__restrict__ ex_off, const int *__restrict__ ex_j,
                                          int *__restrict__ cnt, const int *__restrict__ off, int *__restrict__ l,
                                          int64_t cap, int *st)
{
    typedef typename vec4<T>::type T4;
    const T4 *pos = (const T4 *)pos_v;
    int si = 3 * nW + k;
    const RepDev &R = reps[site_rep[si]];
    int ai = site_orig[si];
    T4 xi = pos[si];
    int ci[3], cx[3], cy[3], cz[3];
    cell_of<T>(R, xi.x, xi.y, xi.z, ci);
    int nx = nb_axis_cells(ci[0], R.nc[0], cx), ny = nb_axis_cells(ci[1], R.nc[1], cy),
        nz = nb_axis_cells(ci[2], R.nc[2], cz);
    int n = 0, w = FILL ? off[k] : 0;
    T rl2 = (T)R.rlist2, rw2 = (T)R.rlistw2;
    for (int a = 0; a < nz; ++a)
        for (int b = 0; b < ny; ++b)
            for (int d = 0; d < nx; ++d) {
                int cell = R.cell0 + cx[d] + R.nc[0] * (cy[b] + R.nc[1] * cz[a]);
                for (int p = bin_start[cell]; p < bin_start[cell + 1]; ++p) {
                    T4 oj = pos[3 * p];
                    if (mi_r2<T>(R, xi.x - oj.x, xi.y - oj.y, xi.z - oj.z) < rw2) {
                        for (int t = 0; t < 3; ++t) {
                            int sj = 3 * p + t;
                            if (nb_excluded(ex_off, ex_j, ai, site_orig[sj])) continue;
                            if (FILL) { if (w + n < cap) l[w + n] = sj; }
                            n++;
                        }
                    }
                }
                for (int p = bin_start[ncell + cell]; p < bin_start[ncell + cell + 1]; ++p) {
                    int sj = 3 * nW + (p - nW);
                    if (sj == si) continue;
                    T4 xj = pos[sj];
                    if (mi_r2<T>(R, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z) < rl2) {
                        if (nb_excluded(ex_off, ex_j, ai, site_orig[sj])) continue;
                        if (FILL) { if (w + n < cap) l[w + n] = sj; }
                        n++;
                    }
                }
            }
    if (!FILL) cnt[k] = n;
    else if ((int64_t)w + n > cap) atomicOr(&st[1], NB_DEV_ERR_OVERFLOW);
}

template <typename T, int FILL>
__global__ void k_xlist(int nA, int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                        const int *__restrict__ site_orig, const void *pos_v, const int *__restrict__ bin_start,
                        int ncell, const int *__restrict__ ex_off, const int *__restrict__ ex_j,
                        int *__restrict__ cnt, const int *__restrict__ off, int *__restrict__ l, int64_t cap, int *st)
{
    if (rebuild_off(st)) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nA; k += gridDim.x * blockDim.x)
        xlist_one<T, FILL>(k, nW, reps, site_rep, site_orig, pos_v, bin_start, ncell, ex_off, ex_j, cnt, off, l, cap,
                           st);
}

// exclusive scan of one int per thread over the block; returns the thread's prefix and the
// block total in *tot (all threads)
__device__ __forceinline__ long long block_excl_scan(long long s, long long *warp_sums, long long *tot)
{
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5;
    long long v = s;
    for (int o = 1; o < 32; o <<= 1) {
        long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[w] = v;
    __syncthreads();
    if (w == 0) {
        long long x = lane < (nt >> 5) ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            long long t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        if (lane < (nt >> 5)) warp_sums[lane] = x;
    }
    __syncthreads();
    long long r = v - s + (w > 0 ? warp_sums[w - 1] : 0);
    *tot = warp_sums[(nt >> 5) - 1];
    __syncthreads();
    return r;
}

// three-phase exclusive scan: tile sums, scan of the tile sums, tile scans.  A tile is
// NB_SCAN_PER x 256 consecutive ints; each thread owns NB_SCAN_PER consecutive entries.
#define NB_SCAN_PER 16
#define NB_SCAN_TILE (NB_SCAN_PER * 256)
__global__ void __launch_bounds__(256) k_scan_sums(const int *__restrict__ in, int n, long long *__restrict__ bsum,
                                                   const int *st, int gate)
{
    if (gate && rebuild_off(st)) return;
    __shared__ long long ws[8];
    const int base = blockIdx.x * NB_SCAN_TILE;
    long long s = 0;
    for (int k = threadIdx.x; k < NB_SCAN_TILE; k += 256)
        if (base + k < n) s += in[base + k];
    long long tot;
    block_excl_scan(s, ws, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_top(long long *__restrict__ bsum, int nb, int *__restrict__ out, int n,
                                                   int *total, const int *st, int gate)
{
    if (gate && rebuild_off(st)) return;
    __shared__ long long ws[32];
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += 1024) {
        const int b = b0 + threadIdx.x;
        long long s = b < nb ? bsum[b] : 0, tot;
        long long p = block_excl_scan(s, ws, &tot);
        if (b < nb) bsum[b] = carry + p;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        out[n] = (int)carry;
        if (total) *total = (int)min(carry, (long long)0x7fffffff);
    }
}

__global__ void __launch_bounds__(256) k_scan_tiles(const int *__restrict__ in, int *__restrict__ out, int n,
                                                    const long long *__restrict__ bsum, const int *st, int gate)
{
    if (gate && rebuild_off(st)) return;
    __shared__ long long ws[8];
    const int i0 = blockIdx.x * NB_SCAN_TILE + threadIdx.x * NB_SCAN_PER;
    int v[NB_SCAN_PER];
    long long s = 0;
#pragma unroll
    for (int k = 0; k < NB_SCAN_PER; ++k) {
        v[k] = i0 + k < n ? in[i0 + k] : 0;
        s += v[k];
    }
    long long tot;
    long long p = bsum[blockIdx.x] + block_excl_scan(s, ws, &tot);
#pragma unroll
    for (int k = 0; k < NB_SCAN_PER; ++k) {
        if (i0 + k < n) out[i0 + k] = (int)p;
        p += v[k];
    }
}

// single-CTA exclusive scan for short inputs (no scratch): chunks of 1024 with a carry
__global__ void __launch_bounds__(1024) k_scan_small(const int *__restrict__ in, int *__restrict__ out, int n,
                                                     int *total)
{
    __shared__ long long ws[32];
    long long carry = 0;
    for (int i0 = 0; i0 < n; i0 += 1024) {
        const int i = i0 + threadIdx.x;
        long long s = i < n ? in[i] : 0, tot;
        long long p = block_excl_scan(s, ws, &tot);
        if (i < n) out[i] = (int)(carry + p);
        carry += tot;
    }
    if (threadIdx.x == 0) {
        out[n] = (int)carry;
        if (total) *total = (int)min(carry, (long long)0x7fffffff);
    }
}

// out[0..n] = exclusive prefix sums of in[0..n), out[n] = total (also to *total when given);
// gate: skip unless the rebuild flag is set
void nb_scan(NbCtx *c, const int *in, int *out, int n, int *total, int gate)
{
    const int nb = std::max(1, (n + NB_SCAN_TILE - 1) / NB_SCAN_TILE);
    cudaStream_t s = c->stream;
    k_scan_sums<<<nb, 256, 0, s>>>(in, n, c->d_scan_tmp, c->d_status, gate);
    k_scan_top<<<1, 1024, 0, s>>>(c->d_scan_tmp, nb, out, n, total, c->d_status, gate);
    k_scan_tiles<<<nb, 256, 0, s>>>(in, out, n, c->d_scan_tmp, c->d_status, gate);
    c->launches += 3;
}

// Reference water of each replica for the FP32 water exclusion energies (water_intra_f):
// squared O-H and H-H distances t0 of the replica's first water (rounded to FP32), its three
// exclusion energies -qq erf(alpha r)/r in FP64 (cdie_ewald.f:117-199), and the quotient of
// the erf(x)/x series in r^2, sum_n (-1)^n (alpha^2 r^2)^n / (n! (2n+1)) to n = 8, by
// (r^2 - t0).  Runs with the list build; needs every water to carry the replica's water
// charges (wsame) and (alpha 2.2 Å)^2 <= 1, where 2.2 Å bounds H-H of a water whose sites
// lie within rwat of its oxygen (the series then converges to 1e-8).
__global__ void k_wref(int nrep, RepDev *__restrict__ reps, const double *__restrict__ coor, const int *st)
{
    if (rebuild_off(st)) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrep) return;
    RepDev &R = reps[r];
    R.wref = 0;
    const double al = R.alphad;
    if (!R.has_water || !R.wsame || R.wfirst < 0 || al * al * 4.84 > 1.0) return;
    const double *x = coor + 3 * (size_t)R.wfirst;
    double t[2] = {0.0, 0.0};
    for (int d = 0; d < 3; ++d) {
        t[0] += (x[3 + d] - x[d]) * (x[3 + d] - x[d]);
        t[1] += (x[6 + d] - x[3 + d]) * (x[6 + d] - x[3 + d]);
    }
    if (!(t[0] > 1e-4 && t[1] > 1e-4 && al * al * t[1] <= 1.0 && al * al * t[0] <= 1.0)) return;
    double e0 = 0.0;
    for (int ty = 0; ty < 2; ++ty) {
        const float t0 = (float)t[ty];
        const double td = (double)t0, rr = sqrt(td), qq = R.qqd[1 + ty];
        e0 += (ty == 0 ? 2.0 : 1.0) * (-qq * erf(al * rr) / rr);
        // series coefficients in r^2: a_n = (-1)^n alpha^(2n) / (n! (2n+1))
        double a[9], f = 1.0, p = 1.0;
        for (int n = 0; n <= 8; ++n) {
            if (n > 0) { f *= n; p *= -al * al; }
            a[n] = p / (f * (2 * n + 1));
        }
        // synthetic division by (r^2 - t0): b_7 = a_8, b_(m-1) = a_m + t0 b_m
        double b = a[8];
        R.wq[ty][7] = (float)b;
        for (int m = 7; m >= 1; --m) {
            b = a[m] + td * b;
            R.wq[ty][m - 1] = (float)b;
        }
        R.wt0[ty] = t0;
        R.wcoef[ty] = (float)(-qq * al * NB_TWO_OVER_SQRTPI);
    }
    R.wcorr0 = e0;
    R.wref = 1;
}

template <typename T>
void build_lists_t(NbCtx *c, const double *d_coor)
{
    // Every kernel below exits at once unless the device rebuild flag is set; grids are
    // bounded to one wave (grid-stride loops) so the skipped launches stay short.
    const int B = 256;
    cudaStream_t s = c->stream;
    auto grid = [&](int64_t n, int b) {
        return (int)std::max<int64_t>(1, std::min<int64_t>((n + b - 1) / b, (int64_t)c->nsm * (2048 / b)));
    };
    int nbin = 2 * c->ncell;
    cudaMemsetAsync(c->d_bin_count, 0, sizeof(int) * (nbin + 1), s);
    k_unit_keys<<<grid(c->nunit, B), B, 0, s>>>((int)c->nunit, (int)c->nW, c->ncell, c->d_unit_atom, c->d_unit_rep,
                                                c->d_reps, d_coor, c->d_unit_key, c->d_unit_slot, c->d_bin_count,
                                                c->d_status);
    nb_scan(c, c->d_bin_count, c->d_bin_start, nbin, nullptr, 1);
    k_unit_scatter<<<grid(c->nunit, B), B, 0, s>>>((int)c->nunit, c->d_unit_key, c->d_unit_slot, c->d_bin_start,
                                                   c->d_sorted_unit, c->d_status);
    k_bin_sort<<<grid(nbin, 4), 128, 0, s>>>(nbin, c->d_bin_start, c->d_sorted_unit, c->d_status);
    k_site_build<T><<<grid(c->nunit, B), B, 0, s>>>(
        (int)c->nunit, (int)c->nW, c->d_sorted_unit, c->d_unit_atom, c->d_atom_rep, c->d_aflags, c->d_lj_f,
        c->d_lj_d, c->d_q, c->d_site_orig, c->d_site_of, c->d_site_rep, c->d_site_flags, c->d_site_lj,
        c->d_site_q, c->d_status);
    k_prepare<T><<<grid(c->nW + c->nA, B), B, 0, s>>>((int)c->nW, (int)c->nA, c->d_site_orig, c->d_site_flags,
                                                      c->d_site_q, d_coor, c->d_pos, c->d_woff, c->d_posb, 0.f,
                                                      c->rwat * c->rwat, 1, c->d_status);
    c->launches += 5;
    // water lists with the row entry type of the handle (uint16 when every replica has fewer
    // than 65,536 waters)
    auto water_lists = [&](auto e_tag) {
        typedef decltype(e_tag) E;
        if (c->nW <= 0) return;
        const int gw = grid(c->nW, 128), nt = (int)c->wtiles.size();
        const int gt = (int)std::min<int64_t>(nt, (int64_t)c->nsm * 16);
        int *cnt2 = c->d_count_tmp;
        // W1 rows (both kernels) and W2 counts in one pass; W2 scan and fill after
        k_wlist<T, 0, E><<<gw, 128, 0, s>>>((int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_bin_start,
                                            c->ncell, c->d_wl1_cnt, cnt2, nullptr, c->d_wl1, c->cap_row1, nullptr, 0,
                                            c->d_status);
        if (nt > 0)
            k_wlist_tiled<T, E><<<gt, NB_WTILE, 0, s>>>(nt, c->d_wtiles, c->d_reps, c->d_pos, c->d_wl1_cnt,
                                                        c->d_wl1, c->cap_row1, c->d_status);
        nb_scan(c, cnt2, c->d_wl2_off, (int)c->nW, c->d_status + 3, 1);
        k_wlist<T, 1, E><<<gw, 128, 0, s>>>((int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_bin_start,
                                            c->ncell, nullptr, nullptr, c->d_wl2_off, nullptr, 0, c->d_wl2, c->cap_wl2,
                                            c->d_status);
        c->launches += nt > 0 ? 3 : 2;
    };
    if (c->row16) water_lists((unsigned short)0);
    else water_lists(0);
    if (sizeof(T) == 4 && c->whalf && c->row16) {
        const int nb = (int)c->hblocks.size(), g = std::min(nb, c->nsm * 4);
        (c->hb == 128 ? k_whalf<128> : (c->hb == 512 ? k_whalf<512> : k_whalf<256>))<<<g, c->hb, 0, s>>>(
            nb, c->d_hblocks, c->d_reps, c->d_wl1_cnt, (const unsigned short *)c->d_wl1, c->cap_row1, c->d_hrow,
            c->caph, c->d_hcnt, c->d_jset, c->d_jn, c->jcap, c->d_status);
        c->launches++;
    }
    if (sizeof(T) == 4 && c->nW > 0 && c->water_excl_fast) {
        k_wref<<<(c->nrep + 127) / 128, 128, 0, s>>>(c->nrep, c->d_reps, d_coor, c->d_status);
        c->launches++;
    }
    if (c->nA > 0) {
        const int ga = grid(c->nA, 128);
        k_xlist<T, 0><<<ga, 128, 0, s>>>((int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, c->d_pos,
                                         c->d_bin_start, c->ncell, c->d_ex_off, c->d_ex_j, c->d_count_tmp, nullptr,
                                         nullptr, 0, c->d_status);
        nb_scan(c, c->d_count_tmp, c->d_xl_off, (int)c->nA, c->d_status + 4, 1);
        k_xlist<T, 1><<<ga, 128, 0, s>>>((int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, c->d_pos,
                                         c->d_bin_start, c->ncell, c->d_ex_off, c->d_ex_j, nullptr, c->d_xl_off,
                                         c->d_xl, c->cap_xl, c->d_status);
        c->launches += 2;
    }
}

template <typename T>
void prepare_t(NbCtx *c, const double *d_coor, int check)
{
    const int B = 256;
    float hs = 0.5f * c->skin;
    const int64_t items = c->nW + c->nA;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((items + B - 1) / B, (int64_t)c->nsm * 8));
    k_prepare<T><<<g, B, 0, c->stream>>>((int)c->nW, (int)c->nA, c->d_site_orig, c->d_site_flags, c->d_site_q,
                                         d_coor, c->d_pos, c->d_woff, c->d_posb, check ? hs * hs : 3.0e38f,
                                         c->rwat * c->rwat, 0, c->d_status);
    c->launches += 1;
}

}  // namespace

namespace {
// the rebuild decision of a captured evaluation: the IF node around the list rebuild runs its
// body only when the coordinate preparation (or the host) set the device rebuild flag
__global__ void k_rebuild_cond(cudaGraphConditionalHandle h, const int *st)
{
    cudaGraphSetConditional(h, st[0] != 0 ? 1u : 0u);
}
}  // namespace

void nb_launch_rebuild_cond(NbCtx *c, cudaGraphConditionalHandle h)
{
    k_rebuild_cond<<<1, 1, 0, c->stream>>>(h, c->d_status);
    c->launches++;
}

void nb_launch_build_lists(NbCtx *c, const double *d_coor)
{
    if (c->precision == MOIL_NB_FP64) build_lists_t<double>(c, d_coor);
    else build_lists_t<float>(c, d_coor);
}

void nb_launch_prepare(NbCtx *c, const double *d_coor, int check)
{
    if (c->precision == MOIL_NB_FP64) prepare_t<double>(c, d_coor, check);
    else prepare_t<float>(c, d_coor, check);
}

void nb_exclusive_scan(NbCtx *c, const int *d_in, int *d_out, int n, int *d_total)
{
    // PME z-bins: the three-phase scan when the handle has its tile-sum scratch; one CTA
    // for the allocation-free entry point, which has none
    if (c->d_scan_tmp) {
        nb_scan(c, d_in, d_out, n, d_total, 0);
        return;
    }
    k_scan_small<<<1, 1024, 0, c->stream>>>(d_in, d_out, n, d_total);
    c->launches += 1;
}
