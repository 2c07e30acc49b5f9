// nb_press.cu -- MOIL's pressure analysis terms (analysis/pressure.f, pressON) after an
// evaluation: per replica the diagonal of the molecular virial, split as pressure.f prints it,
//   virXX..ZZ    LJ pairs (pot/watwat_ewald.f:163-175, pot/cdie_ewald.f:441-453 and
//                555-566, image pairs symm/symwat_ewald.f:161-173, symm/symcdie_ewald.f:151-161)
//   V_PIdirXX..  real-space Ewald Coulomb pairs (watwat_ewald.f:196-204,
//                cdie_ewald.f:412-429, symwat_ewald.f:193-203)
//   V_PIrecXX..  reciprocal sum (pot/ewald_receip.f:799-807; k_press_zvir_f / k_press_zvir in
//                nb_pme.cu)
//   V_PIrelXX..  PME force times the atom's position relative to its molecule's centre of
//                mass (ewald_receip.f:928-933)
// pressure.f:235-238 adds vir + dir + rec - rel; V_PIcor stays zero (its accumulation is
// commented out in cdie_ewald.f:165-170).
//
// Every pair term is F_ij,a (R_I - R_J)_a, R the centres of mass in the image the pair is
// taken in.  R_I - R_J is formed as r_ij - xrel_i + xrel_j from the pair's own minimum-image
// separation and the atoms' positions relative to their centres of mass (xrel), so no centre
// of mass is imaged.  Molecules are made whole by placing each atom at the minimum image of
// its displacement from the previous atom of its molecule (pressure.f joins them along bonds
// with checkANDmove, :985-1010), which needs consecutive atoms of a molecule closer than half
// the box.
//
// The pass reuses the evaluation's lists, site positions, PME binning and PME gradient
// shares, with the pair predicates and the arithmetic of the energy kernels of the handle's
// precision.  On the mixed path the products with the centre-of-mass separations are FP32
// too, summed per thread in FP32 over chunks of NB_PCHUNK list entries and in FP64 across
// chunks (an FP64 operation per pair would cost more than the pair itself: the FP64 pipe is
// 1/64 of FP32); the plain path is FP64 throughout.  Full lists hold every pair twice:
// water-water and atom-atom terms are halved at the end, water-atom pairs are taken from the
// atom's side only with weight two.
#include "nb_internal.h"

namespace {

#define NB_PCHUNK 32

// the pair arithmetic of each precision (as the energy kernels: MUFU rsqrt and the fitted
// erfc in FP32, libdevice in FP64)
template <typename T> struct PressMath;
template <> struct PressMath<float> {
    __device__ static float qq(const RepDev &R, int k) { return R.qq[k]; }
    __device__ static float w12(const RepDev &R) { return R.w12; }
    __device__ static float w6(const RepDev &R) { return R.w6; }
    __device__ static float c2a(const RepDev &R) { return R.c2a; }
    __device__ static float epstmp(const RepDev &R) { return (float)R.epstmp; }
    __device__ static float rsqrt(float x) { return nb_rsqrt_approx(x); }
    __device__ static float erfc_ex(const RepDev &R, float r2, float rinv, float *ex)
    {
        return nb_erfc_ex(R.alpha * r2 * rinv, r2 * R.ex2c, ex);
    }
};
template <> struct PressMath<double> {
    __device__ static double qq(const RepDev &R, int k) { return R.qqd[k]; }
    __device__ static double w12(const RepDev &R) { return R.w12d; }
    __device__ static double w6(const RepDev &R) { return R.w6d; }
    __device__ static double c2a(const RepDev &R) { return NB_TWO_OVER_SQRTPI * R.alphad; }
    __device__ static double epstmp(const RepDev &R) { return R.epstmp; }
    __device__ static double rsqrt(double x) { return ::rsqrt(x); }
    __device__ static double erfc_ex(const RepDev &R, double r2, double rinv, double *ex)
    {
        return nb_erfc_ex(R.alphad * r2 * rinv, 0.0, ex);
    }
};

// minus (dE_LJ/dr)/r of one pair with the LJ switch extension applied
template <typename T>
__device__ __forceinline__ T lj_mdf(const RepDev &R, T r2, T A, T B)
{
    const T s2 = (T)1 / r2, e1 = A - B;
    T df1 = (T)-6 * s2 * (A + e1);
    if (R.lj_switch && r2 > (T)R.ron2) {
        const T dd = (T)R.rv2 - r2;
        const T sw = dd * dd * ((T)R.rv2 + (T)2 * r2 - (T)3 * (T)R.ron2) * (T)R.swden;
        const T dsw = (T)12 * dd * ((T)R.ron2 - r2) * (T)R.swden;
        df1 = df1 * sw + e1 * dsw;
    }
    return -df1;
}

// positions relative to the centres of mass, per caller atom (FP64); one thread per molecule
__global__ void k_press_xrel(int nmol, const int *__restrict__ mol_off, const int *__restrict__ mol_atom,
                             const int *__restrict__ atom_rep, const RepDev *__restrict__ reps,
                             const double *__restrict__ coor, const double *__restrict__ mass,
                             double *__restrict__ xrel)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmol) return;
    const int b = mol_off[m], e = mol_off[m + 1];
    const RepDev &R = reps[atom_rep[mol_atom[b]]];
    double d[3] = {0.0, 0.0, 0.0}, sm[3] = {0.0, 0.0, 0.0}, M = 0.0;
    int prev = mol_atom[b];
    for (int k = b; k < e; ++k) {
        const int a = mol_atom[k];
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            if (k > b) {
                const double t = coor[3 * (size_t)a + x] - coor[3 * (size_t)prev + x];
                d[x] += t - R.Ld[x] * rint(t * R.invLd[x]);
            }
            xrel[3 * (size_t)a + x] = d[x];
            sm[x] += mass[a] * d[x];
        }
        M += mass[a];
        prev = a;
    }
    const double im = M > 0.0 ? 1.0 / M : 0.0;
    const double com[3] = {sm[0] * im, sm[1] * im, sm[2] * im};
    for (int k = b; k < e; ++k) {
        const int a = mol_atom[k];
#pragma unroll
        for (int x = 0; x < 3; ++x) xrel[3 * (size_t)a + x] -= com[x];
    }
}

// the same in site order and the handle's precision, read beside the site positions
template <typename T>
__global__ void k_press_xrel_sites(int nsite, const int *__restrict__ site_orig, const double *__restrict__ xrel,
                                   void *__restrict__ xsite_v)
{
    typedef typename vec4<T>::type T4;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    const double *x = xrel + 3 * (size_t)site_orig[s];
    T4 o;
    o.x = (T)x[0]; o.y = (T)x[1]; o.z = (T)x[2]; o.w = (T)0;
    ((T4 *)xsite_v)[s] = o;
}

// water molecule per thread over its W1 row: 9 Coulomb site pairs and the O-O LJ pair of
// every molecule inside the O-O cutoff (watwat_ewald.f semantics, water charges of RepDev)
template <typename T, typename E>
__global__ void k_press_water(int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                              const void *pos_v, const void *woff_v, const int2 *__restrict__ wl1_cnt,
                              const void *__restrict__ wl1, int cap_row, const void *xsite_v,
                              double *__restrict__ pu)
{
    typedef typename vec4<T>::type T4;
    typedef PressMath<T> M;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nW) return;
    const T4 *pos = (const T4 *)pos_v, *woff = (const T4 *)woff_v, *xsite = (const T4 *)xsite_v;
    const RepDev &R = reps[site_rep[3 * i]];
    const T4 oi = pos[3 * i], h1 = woff[3 * i + 1], h2 = woff[3 * i + 2];
    const T hi[3][3] = {{(T)0, (T)0, (T)0}, {h1.x, h1.y, h1.z}, {h2.x, h2.y, h2.z}};
    const T4 xi = xsite[3 * i];
    const T rmax2 = (T)R.rmax2, rv2 = (T)R.rv2, c2a = M::c2a(R);
    double v[6] = {0, 0, 0, 0, 0, 0};
    T f[6] = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0};
    int cnt = 0;
    const int2 c = wl1_cnt[i];
    const int nn = min(c.x, cap_row), n = min(c.x + c.y, cap_row);
    const E *row = (const E *)wl1 + (size_t)i * cap_row;
    const int base = sizeof(E) == 2 ? R.wat0 : 0;
    for (int q = 0; q < n; ++q) {
        if (q + 32 < nn) nb_prefetch_l1(row + q + 32);   // the row is a DRAM stream per lane
        const int j = base + (int)row[q < nn ? q : cap_row - 1 - (q - nn)];
        const T4 oj = pos[3 * j];
        T d[3] = {oi.x - oj.x, oi.y - oj.y, oi.z - oj.z};
#pragma unroll
        for (int x = 0; x < 3; ++x) d[x] = nb_shift(R, x, d[x], nb_rint(d[x] * rep_invL<T>(R, x)));
        const T r2oo = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2oo > rmax2) continue;
        const T4 j1 = woff[3 * j + 1], j2 = woff[3 * j + 2];
        const T hj[3][3] = {{(T)0, (T)0, (T)0}, {j1.x, j1.y, j1.z}, {j2.x, j2.y, j2.z}};
        const T4 xj = xsite[3 * j];
        const T rm[3] = {d[0] - xi.x + xj.x, d[1] - xi.y + xj.y, d[2] - xi.z + xj.z};
        T fc[3] = {(T)0, (T)0, (T)0};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const T ex = hi[a][0] + d[0] - hj[b][0], ey = hi[a][1] + d[1] - hj[b][1],
                        ez = hi[a][2] + d[2] - hj[b][2];
                const T rr2 = ex * ex + ey * ey + ez * ez, rinv = M::rsqrt(rr2);
                T exv;
                const T erfcv = M::erfc_ex(R, rr2, rinv, &exv);
                const T qq = M::qq(R, (a == 0 && b == 0) ? 0 : ((a == 0 || b == 0) ? 1 : 2));
                const T e = qq * erfcv * rinv;
                const T mdf = (e + qq * c2a * exv) * rinv * rinv;   // minus dE/dr / r
                fc[0] += mdf * ex; fc[1] += mdf * ey; fc[2] += mdf * ez;
            }
#pragma unroll
        for (int x = 0; x < 3; ++x) f[3 + x] += fc[x] * rm[x];
        if (r2oo <= rv2) {
            const T s2 = (T)1 / r2oo, s6 = s2 * s2 * s2;
            const T m1 = lj_mdf<T>(R, r2oo, M::w12(R) * s6 * s6, M::w6(R) * s6);
#pragma unroll
            for (int x = 0; x < 3; ++x) f[x] += m1 * d[x] * rm[x];
        }
        if (++cnt == NB_PCHUNK) {
#pragma unroll
            for (int k = 0; k < 6; ++k) { v[k] += (double)f[k]; f[k] = (T)0; }
            cnt = 0;
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) pu[6 * (size_t)i + k] = v[k] + (double)f[k];
}

// non-water atom per thread over its X list (non-water atoms and water sites), the pair
// predicate of the energy kernels' atom_pair (cdie_ewald.f list1/2/3, nbond.f:115-126)
template <typename T>
__global__ void k_press_atom(int nA, int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                             const void *pos_v, const void *lj_v, const unsigned *__restrict__ sflags,
                             const int *__restrict__ xl_off, const int *__restrict__ xl, int capx, const void *xsite_v,
                             double *__restrict__ pu)
{
    typedef typename vec4<T>::type T4;
    typedef typename cplx<T>::type T2;
    typedef PressMath<T> M;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nA) return;
    const T4 *pos = (const T4 *)pos_v, *xsite = (const T4 *)xsite_v;
    const T2 *lj = (const T2 *)lj_v;
    const int si = 3 * nW + k;
    const RepDev &R = reps[site_rep[si]];
    const T4 xi = pos[si];
    const T2 lji = lj[si];
    const unsigned fi = sflags[si];
    const T4 xa = xsite[si];
    const T rv2 = (T)R.rv2, re2 = (T)R.re2, rmax2 = (T)R.rmax2, c2a = M::c2a(R);
    double v[6] = {0, 0, 0, 0, 0, 0};
    T f[6] = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0};
    int cnt = 0;
    for (int q = min(xl_off[k], capx); q < min(xl_off[k + 1], capx); ++q) {
        const int s = xl[q];
        const T4 xj = pos[s];
        T d[3] = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
#pragma unroll
        for (int x = 0; x < 3; ++x) d[x] = nb_shift(R, x, d[x], nb_rint(d[x] * rep_invL<T>(R, x)));
        const T r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const unsigned fj = sflags[s];
        const bool hr = !R.arith && R.hvdw0 && ((fi | fj) & SF_HTINY) && r2 < re2;
        const bool do_lj = r2 < rv2 && !hr;
        T qq = xi.w * xj.w;
        const bool do_el = r2 < rmax2 && qq != (T)0;
        if (!do_lj && !do_el) continue;
        const T rinv = M::rsqrt(r2), s2 = rinv * rinv;
        T m_el = (T)0, m_lj = (T)0;   // minus (dE/dr)/r of each part
        if (do_el) {
            T exv;
            const T erfcv = M::erfc_ex(R, r2, rinv, &exv);
            qq *= M::epstmp(R);
            m_el = (qq * erfcv * rinv + qq * c2a * exv) * s2;
        }
        if (do_lj) {
            const T2 ljj = lj[s];
            const T s6 = s2 * s2 * s2;
            T A, B;
            if (!R.arith) {
                A = lji.x * ljj.x * s6 * s6;
                B = lji.y * ljj.y * s6;
            } else {
                const T aa = lji.x * ljj.x, sg = (T)0.5 * (lji.y + ljj.y);
                T b1 = sg * sg * sg;
                b1 = b1 * b1;
                B = aa * b1 * s6;
                A = aa * b1 * b1 * s6 * s6;
            }
            m_lj = lj_mdf<T>(R, r2, A, B);
        }
        const T w = s < 3 * nW ? (T)2 : (T)1;   // water partners: this side only
        const T4 xb = xsite[s];
        const T rm[3] = {d[0] - xa.x + xb.x, d[1] - xa.y + xb.y, d[2] - xa.z + xb.z};
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            f[x] += w * m_lj * d[x] * rm[x];
            f[3 + x] += w * m_el * d[x] * rm[x];
        }
        if (++cnt == NB_PCHUNK) {
#pragma unroll
            for (int m = 0; m < 6; ++m) { v[m] += (double)f[m]; f[m] = (T)0; }
            cnt = 0;
        }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) pu[6 * (size_t)(nW + k) + q] = v[q] + (double)f[q];
}

// V_PIrel per site: the PME force (minus the gradient share k_final_grad adds) times xrel
template <typename T>
__global__ void k_press_rel(int nsite, const int *__restrict__ site_rep, const int *__restrict__ site_orig,
                            const RepDev *__restrict__ reps, const void *part_v, const double *__restrict__ q,
                            const void *xsite_v, double *__restrict__ ps)
{
    typedef typename vec4<T>::type T4;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    const RepDev &R = reps[site_rep[s]];
    const int a = site_orig[s];
    const T4 x = ((const T4 *)xsite_v)[s];
    if constexpr (sizeof(T) == 4) {
        // one float4 per site from k_pme_gather_f, scaled by q fc n_d / L_d
        const float4 p = ((const float4 *)part_v)[s];
        const float qs = -(float)q[a];
        ps[3 * (size_t)s] = (double)(qs * R.pme_gs[0] * p.x * x.x);
        ps[3 * (size_t)s + 1] = (double)(qs * R.pme_gs[1] * p.y * x.y);
        ps[3 * (size_t)s + 2] = (double)(qs * R.pme_gs[2] * p.z * x.z);
    } else {
        // four plane slots of three per site from k_plane_inv
        const double *p = (const double *)part_v + 12 * (size_t)s;
        const double qf = q[a] * R.fcd;
        const double sc[3] = {qf * R.n1 * R.invLd[0], qf * R.n2 * R.invLd[1], qf * R.n3 * R.invLd[2]};
        const double xr[3] = {x.x, x.y, x.z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double g = p[d] + p[3 + d] + p[6 + d] + p[9 + d];
            ps[3 * (size_t)s + d] = -sc[d] * g * xr[d];
        }
    }
}

// per replica, fixed order: strided slots per thread, then a halving tree
#define NB_PR_THREADS 256
__global__ void __launch_bounds__(NB_PR_THREADS) k_press_reduce(int nW, const RepDev *__restrict__ reps,
                                                               const double *__restrict__ pu,
                                                               const double *__restrict__ ps,
                                                               const double *__restrict__ v_col,
                                                               const int *__restrict__ col_begin,
                                                               double *__restrict__ out)
{
    __shared__ double red[12][NB_PR_THREADS];
    const int r = blockIdx.x, t = threadIdx.x;
    const RepDev &R = reps[r];
    double acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = 0.0;
    const int u0[2] = {R.wat0, nW + R.oth0}, nu[2] = {R.nwat, R.noth};
    const int s0[2] = {3 * R.wat0, 3 * nW + R.oth0}, ns[2] = {3 * R.nwat, R.noth};
    for (int p = 0; p < 2; ++p) {
        for (int u = t; u < nu[p]; u += NB_PR_THREADS) {
            const double *v = pu + 6 * (size_t)(u0[p] + u);
#pragma unroll
            for (int k = 0; k < 6; ++k) acc[k] += v[k];
        }
        for (int u = t; u < ns[p]; u += NB_PR_THREADS) {
            const double *v = ps + 3 * (size_t)(s0[p] + u);
#pragma unroll
            for (int k = 0; k < 3; ++k) acc[9 + k] += v[k];
        }
    }
    for (int w = col_begin[r] + t; w < col_begin[r + 1]; w += NB_PR_THREADS) {
#pragma unroll
        for (int k = 0; k < 3; ++k) acc[6 + k] += v_col[3 * (size_t)w + k];
    }
#pragma unroll
    for (int k = 0; k < 12; ++k) red[k][t] = acc[k];
    __syncthreads();
    for (int h = NB_PR_THREADS / 2; h > 0; h >>= 1) {
        if (t < h)
#pragma unroll
            for (int k = 0; k < 12; ++k) red[k][t] += red[k][t + h];
        __syncthreads();
    }
    if (t < 12) out[12 * (size_t)r + t] = (t < 9 ? 0.5 : 1.0) * red[t][0];
}

template <typename T>
void pressure_t(NbCtx *c, const double *d_coor, double *d_out)
{
    cudaStream_t s = c->stream;
    const int B = 128;
    if (c->nmol > 0)
        k_press_xrel<<<(c->nmol + B - 1) / B, B, 0, s>>>(c->nmol, c->d_mol_off, c->d_mol_atom, c->d_atom_rep,
                                                        c->d_reps, d_coor, c->d_mass, c->d_xrel);
    k_press_xrel_sites<T><<<(int)((c->nsite + 255) / 256), 256, 0, s>>>((int)c->nsite, c->d_site_orig, c->d_xrel,
                                                                      c->d_xsite);
    if (c->nW > 0)
        (c->row16 ? k_press_water<T, unsigned short> : k_press_water<T, int>)<<<(int)((c->nW + B - 1) / B), B, 0, s>>>(
            (int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_woff, c->d_wl1_cnt, c->d_wl1, c->cap_row1,
            c->d_xsite, c->d_press_unit);
    if (c->nA > 0)
        k_press_atom<T><<<(int)((c->nA + B - 1) / B), B, 0, s>>>(
            (int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_site_lj, c->d_site_flags, c->d_xl_off,
            c->d_xl, cap_int(c->cap_xl), c->d_xsite, c->d_press_unit);
    k_press_rel<T><<<(int)((c->nsite + 255) / 256), 256, 0, s>>>((int)c->nsite, c->d_site_rep, c->d_site_orig,
                                                               c->d_reps, c->d_part, c->d_q, c->d_xsite,
                                                               c->d_press_site);
}

}  // namespace

void nb_launch_pme_virial(NbCtx *c, void *grid, double *v_col);

int nb_pressure(NbCtx *c, const double *d_coor, double *d_out)
{
    if (c->precision == MOIL_NB_FP64) pressure_t<double>(c, d_coor, d_out);
    else pressure_t<float>(c, d_coor, d_out);
    nb_launch_pme_virial(c, c->d_press_grid, c->d_press_col);
    k_press_reduce<<<c->nrep, NB_PR_THREADS, 0, c->stream>>>((int)c->nW, c->d_reps, c->d_press_unit,
                                                             c->d_press_site, c->d_press_col, c->d_col_begin, d_out);
    NB_CUDA_OK(c, cudaGetLastError());
    return MOIL_NB_OK;
}
