// nb_lists.cu -- list rebuild: the GPU replacement of squeeze()/nbondm()/nbond()/syminit().
//
// MOIL builds an O(M^2) monomer list (pot/nbondm.f:143-210), atom lists with exclusion and
// hydrogen filters (pot/nbond.f:54-157) and 13 image-translation lists (symm/nbmsym.f,
// symm/nbsym.f).  Here the same pair set comes from a cell list with minimum-image
// distances (identical for cutoff <= L/2):
//   units     : water molecules (anchor O, pot/nbondm.f:81-86) and non-water atoms
//   sort      : counting sort of units by (class, replica, cell), ties by unit id
//   lists     : W1  water i -> water j   (O-O < rmax + skin)             full list
//               W2  water i -> non-water site j (O-x < rmax + skin + rwat)
//               X   non-water i -> any site j (exclusions removed, as pot/nbond.f:95-103)
// Every list is a full (both-direction) CSR list so each lane owns its gradient outright.
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
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nunit) return;
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

__global__ void k_unit_scatter(int nunit, const int *__restrict__ key, const int *__restrict__ slot,
                               const int *__restrict__ start, int *__restrict__ sorted, const int *st)
{
    if (rebuild_off(st)) return;
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nunit) return;
    sorted[start[key[u]] + slot[u]] = u;
}

// deterministic order inside a bin: ascending unit id (insertion sort, bins are short)
__global__ void k_bin_sort(int nbin, const int *__restrict__ start, int *__restrict__ sorted, const int *st)
{
    if (rebuild_off(st)) return;
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbin) return;
    int lo = start[b], hi = start[b + 1];
    for (int i = lo + 1; i < hi; ++i) {
        int v = sorted[i], j = i - 1;
        while (j >= lo && sorted[j] > v) { sorted[j + 1] = sorted[j]; --j; }
        sorted[j + 1] = v;
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
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nunit) return;
    int u = sorted[p];
    int a0 = unit_atom[u];
    int s0, ns;
    if (p < nW) { s0 = 3 * p; ns = 3; } else { s0 = 3 * nW + (p - nW); ns = 1; }
    typedef typename cplx<T>::type T2;
    T2 *site_lj = (T2 *)site_lj_v;
    T *site_q = (T *)site_q_v;
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

// 3. per-evaluation coordinate conversion into site order; displacement check
template <typename T>
__global__ void k_prepare(int nsite, int nW, const int *__restrict__ site_orig, const int *__restrict__ site_rep,
                          const unsigned *__restrict__ site_flags, const double *__restrict__ q,
                          const RepDev *__restrict__ reps, const double *__restrict__ coor, void *pos_v,
                          void *woff_v, float4 *__restrict__ posb, float half_skin2, float rwat2, int snapshot,
                          int *st)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    if (snapshot && rebuild_off(st)) return;
    typedef typename vec4<T>::type T4;
    int a = site_orig[s];
    double x = coor[3 * (size_t)a], y = coor[3 * (size_t)a + 1], z = coor[3 * (size_t)a + 2];
    if (!(x == x && y == y && z == z) || fabs(x) > 1e7 || fabs(y) > 1e7 || fabs(z) > 1e7) {
        atomicOr(&st[1], NB_DEV_ERR_NAN);
        x = y = z = 0.0;
    }
    unsigned f = site_flags[s];
    T qe = (f & SF_CHARGED) ? (T)q[a] : (T)0;
    T4 p;
    p.x = (T)x; p.y = (T)y; p.z = (T)z; p.w = qe;
    ((T4 *)pos_v)[s] = p;
    float4 pf = make_float4((float)x, (float)y, (float)z, 0.f);
    if (snapshot) {
        posb[s] = pf;
    } else {
        // lists stay valid while no site moved more than skin/2 since the build
        float4 b = posb[s];
        float dx = pf.x - b.x, dy = pf.y - b.y, dz = pf.z - b.z;
        if (dx * dx + dy * dy + dz * dz > half_skin2) atomicOr(&st[0], 1);
    }
    if (s < 3 * nW && (s % 3) != 0) {
        // water sites must stay within rwat of their oxygen (list radius assumption)
        int o = site_orig[s - (s % 3)];
        double ox = coor[3 * (size_t)o], oy = coor[3 * (size_t)o + 1], oz = coor[3 * (size_t)o + 2];
        double d2 = (x - ox) * (x - ox) + (y - oy) * (y - oy) + (z - oz) * (z - oz);
        if (d2 > rwat2) atomicOr(&st[1], NB_DEV_ERR_RWAT);
        // H offset from its O, formed in FP64 so the water kernel's site displacements
        // inherit no extra rounding from absolute FP32 positions
        T4 off;
        off.x = (T)(x - ox); off.y = (T)(y - oy); off.z = (T)(z - oz); off.w = (T)0;
        ((T4 *)woff_v)[2 * (s / 3) + (s % 3) - 1] = off;
    }
    (void)site_rep;
    (void)reps;
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

// 4. water lists W1 (water j) and W2 (non-water sites); FILL = 0 counts, 1 writes
template <typename T, int FILL>
__global__ void k_wlist(int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep, const void *pos_v,
                        const int *__restrict__ bin_start, int ncell, const int *__restrict__ sorted,
                        int *__restrict__ cnt1, int *__restrict__ cnt2, int *__restrict__ cntn,
                        const int *__restrict__ off1, const int *__restrict__ off2, int *__restrict__ l1,
                        int *__restrict__ l2, int64_t cap1, int64_t cap2, int *st)
{
    // W1 entries are stored in two groups: molecules already inside the cutoff at build
    // time first, skin-only molecules after them, so lanes of a warp stay converged
    if (rebuild_off(st)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nW) return;
    typedef typename vec4<T>::type T4;
    const T4 *pos = (const T4 *)pos_v;
    const RepDev &R = reps[site_rep[3 * i]];
    T4 oi = pos[3 * i];
    int ci[3], cx[3], cy[3], cz[3];
    cell_of<T>(R, oi.x, oi.y, oi.z, ci);
    int nx = nb_axis_cells(ci[0], R.nc[0], cx), ny = nb_axis_cells(ci[1], R.nc[1], cy),
        nz = nb_axis_cells(ci[2], R.nc[2], cz);
    int n1 = 0, n2 = 0, nn = 0;
    int w1 = FILL ? off1[i] : 0, w2 = FILL ? off2[i] : 0, wf = FILL ? off1[i] + cntn[i] : 0;
    T rl2 = (T)R.rlist2, rw2 = (T)R.rlistw2, rc2 = (T)R.rmax2;
    int nW_i = nW;
    for (int a = 0; a < nz; ++a)
        for (int b = 0; b < ny; ++b)
            for (int d = 0; d < nx; ++d) {
                int cell = R.cell0 + cx[d] + R.nc[0] * (cy[b] + R.nc[1] * cz[a]);
                // waters in the cell: sorted positions [bin_start[cell], bin_start[cell+1])
                for (int p = bin_start[cell]; p < bin_start[cell + 1]; ++p) {
                    if (p == i) continue;
                    T4 oj = pos[3 * p];
                    T r2 = mi_r2<T>(R, oi.x - oj.x, oi.y - oj.y, oi.z - oj.z);
                    if (r2 < rl2) {
                        bool near = r2 <= rc2;
                        if (FILL) {
                            int at = near ? w1 + nn : wf + (n1 - nn);
                            if (at < cap1) l1[at] = p;
                        }
                        nn += near;
                        n1++;
                    }
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
    if (!FILL) { cnt1[i] = n1; cnt2[i] = n2; cntn[i] = nn; }
    else if ((int64_t)w1 + n1 > cap1 || (int64_t)w2 + n2 > cap2) atomicOr(&st[1], NB_DEV_ERR_OVERFLOW);
}

// 5. non-water list X: every site j within reach, exclusions removed
template <typename T, int FILL>
__global__ void k_xlist(int nA, int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                        const int *__restrict__ site_orig, const void *pos_v, const int *__restrict__ bin_start,
                        int ncell, const int *__restrict__ ex_off, const int *__restrict__ ex_j,
                        int *__restrict__ cnt, const int *__restrict__ off, int *__restrict__ l, int64_t cap, int *st)
{
    if (rebuild_off(st)) return;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nA) return;
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

// single-CTA exclusive scan (n up to a few million); total -> *total; skips when rebuild is off
__global__ void k_scan(const int *__restrict__ in, int *__restrict__ out, int n, int *total, const int *st,
                       int gate)
{
    if (gate && rebuild_off(st)) return;
    __shared__ long long warp_sums[32];
    __shared__ long long carry_s;
    int tid = threadIdx.x, nt = blockDim.x;
    int chunk = (n + nt - 1) / nt;
    int lo = tid * chunk, hi = min(n, lo + chunk);
    long long s = 0;
    for (int i = lo; i < hi; ++i) s += in[i];
    // block exclusive scan of s
    long long v = s;
    int lane = tid & 31, w = tid >> 5;
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
        if (lane == 31) carry_s = x;
    }
    __syncthreads();
    long long base = v - s + (w > 0 ? warp_sums[w - 1] : 0);
    for (int i = lo; i < hi; ++i) {
        out[i] = (int)base;
        base += in[i];
    }
    if (tid == nt - 1) {
        out[n] = (int)(base);
        if (total) *total = (int)min(base, (long long)0x7fffffff);
    }
    (void)carry_s;
}

template <typename T>
void build_lists_t(NbCtx *c, const double *d_coor)
{
    const int B = 256;
    cudaStream_t s = c->stream;
    int nbin = 2 * c->ncell;
    cudaMemsetAsync(c->d_bin_count, 0, sizeof(int) * (nbin + 1), s);
    // histogram is gated by the rebuild flag inside the kernel; the memset is harmless
    k_unit_keys<<<(int)((c->nunit + B - 1) / B), B, 0, s>>>((int)c->nunit, (int)c->nW, c->ncell, c->d_unit_atom,
                                                           c->d_unit_rep, c->d_reps, d_coor, c->d_unit_key,
                                                           c->d_unit_slot, c->d_bin_count, c->d_status);
    k_scan<<<1, 1024, 0, s>>>(c->d_bin_count, c->d_bin_start, nbin, nullptr, c->d_status, 1);
    k_unit_scatter<<<(int)((c->nunit + B - 1) / B), B, 0, s>>>((int)c->nunit, c->d_unit_key, c->d_unit_slot,
                                                              c->d_bin_start, c->d_sorted_unit, c->d_status);
    k_bin_sort<<<(nbin + B - 1) / B, B, 0, s>>>(nbin, c->d_bin_start, c->d_sorted_unit, c->d_status);
    k_site_build<T><<<(int)((c->nunit + B - 1) / B), B, 0, s>>>(
        (int)c->nunit, (int)c->nW, c->d_sorted_unit, c->d_unit_atom, c->d_atom_rep, c->d_aflags, c->d_lj_f,
        c->d_lj_d, c->d_q, c->d_site_orig, c->d_site_of, c->d_site_rep, c->d_site_flags, c->d_site_lj,
        c->d_site_q, c->d_status);
    k_prepare<T><<<(int)((c->nsite + B - 1) / B), B, 0, s>>>(
        (int)c->nsite, (int)c->nW, c->d_site_orig, c->d_site_rep, c->d_site_flags, c->d_q, c->d_reps, d_coor,
        c->d_pos, c->d_woff, c->d_posb, 0.f, c->rwat * c->rwat, 1, c->d_status);
    c->launches += 6;
    if (c->nW > 0) {
        int nb = (int)((c->nW + 127) / 128);
        k_wlist<T, 0><<<nb, 128, 0, s>>>((int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_bin_start, c->ncell,
                                         c->d_sorted_unit, c->d_count_tmp, c->d_count_tmp + c->nW + 1,
                                         c->d_count_tmp + 2 * (c->nW + 1), nullptr, nullptr, nullptr, nullptr, 0, 0,
                                         c->d_status);
        k_scan<<<1, 1024, 0, s>>>(c->d_count_tmp, c->d_wl1_off, (int)c->nW, c->d_status + 2, c->d_status, 1);
        k_scan<<<1, 1024, 0, s>>>(c->d_count_tmp + c->nW + 1, c->d_wl2_off, (int)c->nW, c->d_status + 3,
                                  c->d_status, 1);
        k_wlist<T, 1><<<nb, 128, 0, s>>>((int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_bin_start, c->ncell,
                                         c->d_sorted_unit, nullptr, nullptr, c->d_count_tmp + 2 * (c->nW + 1),
                                         c->d_wl1_off, c->d_wl2_off, c->d_wl1, c->d_wl2, c->cap_wl1, c->cap_wl2,
                                         c->d_status);
        c->launches += 4;
    }
    if (c->nA > 0) {
        int nb = (int)((c->nA + 127) / 128);
        k_xlist<T, 0><<<nb, 128, 0, s>>>((int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, c->d_pos,
                                         c->d_bin_start, c->ncell, c->d_ex_off, c->d_ex_j, c->d_count_tmp, nullptr,
                                         nullptr, 0, c->d_status);
        k_scan<<<1, 1024, 0, s>>>(c->d_count_tmp, c->d_xl_off, (int)c->nA, c->d_status + 4, c->d_status, 1);
        k_xlist<T, 1><<<nb, 128, 0, s>>>((int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, c->d_pos,
                                         c->d_bin_start, c->ncell, c->d_ex_off, c->d_ex_j, nullptr, c->d_xl_off,
                                         c->d_xl, c->cap_xl, c->d_status);
        c->launches += 3;
    }
}

template <typename T>
void prepare_t(NbCtx *c, const double *d_coor, int check)
{
    const int B = 256;
    float hs = 0.5f * c->skin;
    k_prepare<T><<<(int)((c->nsite + B - 1) / B), B, 0, c->stream>>>(
        (int)c->nsite, (int)c->nW, c->d_site_orig, c->d_site_rep, c->d_site_flags, c->d_q, c->d_reps, d_coor,
        c->d_pos, c->d_woff, c->d_posb, check ? hs * hs : 3.0e38f, c->rwat * c->rwat, 0, c->d_status);
    c->launches += 1;
}

}  // namespace

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
    k_scan<<<1, 1024, 0, c->stream>>>(d_in, d_out, n, d_total, c->d_status, 0);
    c->launches += 1;
}
