// nb_adjoint.cu -- parameter derivatives of the nonbonded energy: dE/dq, dE/deps and
// dE/dsigma per atom (moil_nb_adjoint).  MOIL computes none of them; the oracle's
// ora_adjoint_mi is the reference, itself checked against finite differences.
//
// One evaluation (moil_nb_eval semantics) leaves the lists, the site-ordered positions and
// the PME grid on the device (the real potential planes on the mixed path, the convolved
// spectrum on the plain path, whose inverse plane kernel then gives each site's potential
// shares); these kernels then accumulate, in FP64:
//   dE/dq_i     = sum over i's real-space partners of k q_j erfc(alpha r)/r
//               - sum over i's excluded partners of k q_j erf(alpha r)/r
//               + 1-4 Coulomb p14(3)/(q_i r) + fc * sum(theta * potential grid)
//               - 2 alpha/sqrt(pi) k q_i                      (k = kofdie/eps, fc = sqrt(k))
//   dE/deps_i   = sum over i's LJ pairs of (A - B) / (2 eps_i)     (A ~ r^-12, B ~ r^-6 parts)
//   dE/dsigma_i = sum over i's LJ pairs of (6A - 3B) / sigma_i   (geometric: sigma_ij^6 =
//                 sigma_i^3 sigma_j^3), or / sigma_ij with sigma_ij = (sigma_i + sigma_j)/2
//                 (arithmetic)
// with eps and sigma decoded from MOIL's epsgm encoding (connect/fillpt.f:136-184).  The
// pair predicates are the energy kernels' (MOIL's, pot/watwat_ewald.f, pot/cdie_ewald.f);
// water-water Coulomb uses each site's own charge (MOIL's water kernel the last water's,
// the same for identical waters).  The LJ switch extension is not differentiated.
#include "nb_internal.h"

namespace {

// geometric: epsgm12 = 2 sqrt(eps) sigma^6, epsgm6 = 2 sqrt(eps) sigma^3;
// arithmetic: epsgm12 = 2 sqrt(eps), epsgm6 = sigma
__device__ __forceinline__ void lj_decode(int arith, double e12, double e6, double &eps, double &sig)
{
    if (arith) {
        eps = 0.25 * e12 * e12;
        sig = e6;
    } else if (e12 > 0.0 && e6 > 0.0) {
        const double se = e6 * e6 / (2.0 * e12);
        sig = cbrt(e12 / e6);
        eps = se * se;
    } else {
        eps = 0.0;
        sig = 0.0;
    }
}

// the pair's LJ energy parts a (r^-12) and b (r^-6) into atom i's derivatives
__device__ __forceinline__ void lj_adj(int arith, double a, double b, double eps_i, double sig_i, double sig_j,
                                       double &de, double &ds)
{
    const double e = a - b, g = 6.0 * a - 3.0 * b;
    if (eps_i > 0.0) de += e / (2.0 * eps_i);
    if (!arith) {
        if (sig_i > 0.0) ds += g / sig_i;
    } else {
        const double sij = 0.5 * (sig_i + sig_j);
        if (sij > 0.0) ds += g / sij;
    }
}

// LJ parts of a non-water pair (cdie_ewald.f:377-383 geometric, :432-472 arithmetic)
__device__ __forceinline__ void lj_parts(int arith, double e12i, double e6i, double e12j, double e6j, double s2,
                                         double &a, double &b)
{
    const double s6 = s2 * s2 * s2;
    if (!arith) {
        a = e12i * e12j * s6 * s6;
        b = e6i * e6j * s6;
    } else {
        const double aa = e12i * e12j, sg = 0.5 * (e6i + e6j);
        double b1 = sg * sg * sg;
        b1 = b1 * b1;
        b = aa * b1 * s6;
        a = aa * b1 * b1 * s6 * s6;
    }
}

template <typename T>
__device__ __forceinline__ double2 lj_of(const void *lj_v, int s)
{
    typedef typename cplx<T>::type T2;
    const T2 v = ((const T2 *)lj_v)[s];
    return make_double2((double)v.x, (double)v.y);
}

// one non-water-semantics site pair (atom_pair of the energy kernels) into site i's sums
template <typename T>
__device__ __forceinline__ void atom_pair_adj(const RepDev &R, double r2, double qi, double qj, double2 lji,
                                              double2 ljj, unsigned fi, unsigned fj, double &phi, double &de,
                                              double &ds)
{
    const bool hr = !R.arith && R.hvdw0 && ((fi | fj) & SF_HTINY) && r2 < (double)R.re2;
    const bool lj = r2 < (double)R.rv2 && !hr;
    const bool el = r2 < (double)R.rmax2 && qi * qj != 0.0;
    if (el) {
        const double r = sqrt(r2);
        phi += R.epstmp * qj * erfc(R.alphad * r) / r;
    }
    if (lj) {
        double a, b, ei, si, ej, sj;
        lj_parts(R.arith, lji.x, lji.y, ljj.x, ljj.y, 1.0 / r2, a, b);
        lj_decode(R.arith, lji.x, lji.y, ei, si);
        lj_decode(R.arith, ljj.x, ljj.y, ej, sj);
        lj_adj(R.arith, a, b, ei, si, sj, de, ds);
    }
}

// water molecule per thread: W1 (nine site pairs per molecule pair) and W2
template <typename T, typename E>
__global__ void k_adj_water(int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                            const int *__restrict__ site_orig, const void *pos_v, const void *woff_v,
                            const void *lj_v, const unsigned *__restrict__ sflags, const int2 *__restrict__ wl1_cnt,
                            const void *__restrict__ wl1, int cap_row, const int *__restrict__ wl2_off,
                            const int *__restrict__ wl2, int cap2, double *__restrict__ dq, double *__restrict__ de,
                            double *__restrict__ ds)
{
    typedef typename vec4<T>::type T4;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nW) return;
    const T4 *pos = (const T4 *)pos_v;
    const T4 *woff = (const T4 *)woff_v;
    const RepDev &R = reps[site_rep[3 * i]];
    const T4 oi = pos[3 * i];
    const T4 h1 = woff[3 * i + 1], h2 = woff[3 * i + 2];
    const T hi[3][3] = {{(T)0, (T)0, (T)0}, {h1.x, h1.y, h1.z}, {h2.x, h2.y, h2.z}};
    double phi[3] = {0, 0, 0}, dE[3] = {0, 0, 0}, dS[3] = {0, 0, 0};
    double epsO, sigO;
    const double2 ljO = lj_of<T>(lj_v, 3 * i);
    lj_decode(R.arith, ljO.x, ljO.y, epsO, sigO);
    const int2 c = wl1_cnt[i];
    const int nn = min(c.x, cap_row), n = min(c.x + c.y, cap_row);
    const E *row = (const E *)wl1 + (size_t)i * cap_row;
    const int base = sizeof(E) == 2 ? R.wat0 : 0;   // uint16 entries: offsets from the replica's first water
    for (int v = 0; v < n; ++v) {
        const int j = base + (int)row[v < nn ? v : cap_row - 1 - (v - nn)];
        const T4 oj = pos[3 * j];
        T dx = oi.x - oj.x, dy = oi.y - oj.y, dz = oi.z - oj.z;
        const T nx = nb_rint(dx * rep_invL<T>(R, 0)), ny = nb_rint(dy * rep_invL<T>(R, 1)),
                nz = nb_rint(dz * rep_invL<T>(R, 2));
        dx = nb_shift(R, 0, dx, nx);
        dy = nb_shift(R, 1, dy, ny);
        dz = nb_shift(R, 2, dz, nz);
        const T r2oo = dx * dx + dy * dy + dz * dz;
        if (r2oo > (T)R.rmax2) continue;
        const T4 j1 = woff[3 * j + 1], j2 = woff[3 * j + 2];
        const T hj[3][3] = {{(T)0, (T)0, (T)0}, {j1.x, j1.y, j1.z}, {j2.x, j2.y, j2.z}};
        const double qj[3] = {(double)oj.w, (double)pos[3 * j + 1].w, (double)pos[3 * j + 2].w};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const double ex = (double)(hi[a][0] + dx - hj[b][0]), ey = (double)(hi[a][1] + dy - hj[b][1]),
                             ez = (double)(hi[a][2] + dz - hj[b][2]);
                const double r = sqrt(ex * ex + ey * ey + ez * ez);
                phi[a] += R.epstmp * qj[b] * erfc(R.alphad * r) / r;
            }
        if (r2oo <= (T)R.rv2) {
            const double s2 = 1.0 / (double)r2oo, s6 = s2 * s2 * s2;
            double ej, sj;
            const double2 ljj = lj_of<T>(lj_v, 3 * j);
            lj_decode(R.arith, ljj.x, ljj.y, ej, sj);
            lj_adj(R.arith, R.w12d * s6 * s6, R.w6d * s6, epsO, sigO, sj, dE[0], dS[0]);
        }
    }
    for (int k = min(wl2_off[i], cap2); k < min(wl2_off[i + 1], cap2); ++k) {
        const int s = wl2[k];
        const T4 xj = pos[s];
        const double2 ljj = lj_of<T>(lj_v, s);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const T4 xi = pos[3 * i + a];
            T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            dx = nb_shift(R, 0, dx, nb_rint(dx * rep_invL<T>(R, 0)));
            dy = nb_shift(R, 1, dy, nb_rint(dy * rep_invL<T>(R, 1)));
            dz = nb_shift(R, 2, dz, nb_rint(dz * rep_invL<T>(R, 2)));
            atom_pair_adj<T>(R, (double)(dx * dx + dy * dy + dz * dz), (double)xi.w, (double)xj.w,
                             lj_of<T>(lj_v, 3 * i + a), ljj, sflags[3 * i + a], sflags[s], phi[a], dE[a], dS[a]);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int o = site_orig[3 * i + a];
        dq[o] = phi[a];
        de[o] = dE[a];
        ds[o] = dS[a];
    }
}

// non-water atom per thread over its X list
template <typename T>
__global__ void k_adj_atom(int nA, int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                           const int *__restrict__ site_orig, const void *pos_v, const void *lj_v,
                           const unsigned *__restrict__ sflags, const int *__restrict__ xl_off,
                           const int *__restrict__ xl, int capx, double *__restrict__ dq, double *__restrict__ de,
                           double *__restrict__ ds)
{
    typedef typename vec4<T>::type T4;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nA) return;
    const T4 *pos = (const T4 *)pos_v;
    const int si = 3 * nW + k;
    const RepDev &R = reps[site_rep[si]];
    const T4 xi = pos[si];
    const double2 lji = lj_of<T>(lj_v, si);
    double phi = 0, dE = 0, dS = 0;
    for (int q = min(xl_off[k], capx); q < min(xl_off[k + 1], capx); ++q) {
        const int s = xl[q];
        const T4 xj = pos[s];
        T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        dx = nb_shift(R, 0, dx, nb_rint(dx * rep_invL<T>(R, 0)));
        dy = nb_shift(R, 1, dy, nb_rint(dy * rep_invL<T>(R, 1)));
        dz = nb_shift(R, 2, dz, nb_rint(dz * rep_invL<T>(R, 2)));
        atom_pair_adj<T>(R, (double)(dx * dx + dy * dy + dz * dz), (double)xi.w, (double)xj.w, lji,
                         lj_of<T>(lj_v, s), sflags[si], sflags[s], phi, dE, dS);
    }
    const int o = site_orig[si];
    dq[o] = phi;
    de[o] = dE;
    ds[o] = dS;
}

// ---------------------------------------------------------------------------------
// Mixed path: the same sums with FP32 pair arithmetic (the energy kernels' erfc fit and a
// Newton-refined reciprocal square root), summed per site in FP32 over chunks of CHUNK_ADJ list
// entries and flushed into FP64 -- the FP64 pipe of this GPU is a small fraction of the FP32
// one, so per-pair FP64 erfc, square roots and divisions would dominate.  k = kofdie/eps is
// applied to the FP64 potential sums at the end.
#define CHUNK_ADJ 64

// 1/sqrt(r2) to about an ulp: the approximate MUFU value and one Newton step
__device__ __forceinline__ float adj_rsqrt(float r2)
{
    const float y = nb_rsqrt_approx(r2);
    return fmaf(-0.5f * y, fmaf(r2, y * y, -1.f), y);
}

// eps and sigma from the epsgm encoding in FP32 (as lj_decode)
__device__ __forceinline__ void lj_decode_f(int arith, float e12, float e6, float &eps, float &sig)
{
    if (arith) {
        eps = 0.25f * e12 * e12;
        sig = e6;
    } else if (e12 > 0.f && e6 > 0.f) {
        const float se = e6 * e6 / (2.f * e12);
        sig = cbrtf(e12 / e6);
        eps = se * se;
    } else {
        eps = 0.f;
        sig = 0.f;
    }
}

// one non-water-semantics site pair (atom_pair of the energy kernels): q_j erfc(alpha r)/r into
// phi (k applied later), the LJ parts into de, ds of site i (1/(2 eps_i), 1/sigma_i given)
__device__ __forceinline__ void atom_pair_adj_f(const RepDev &R, float r2, float qi, float qj, float2 lji,
                                                float2 ljj, unsigned fi, unsigned fj, float inv2e_i, float sig_i,
                                                float &phi, float &de, float &ds)
{
    const bool hr = !R.arith && R.hvdw0 && ((fi | fj) & SF_HTINY) && r2 < R.re2;
    const bool lj = r2 < R.rv2 && !hr;
    const bool el = r2 < R.rmax2 && qi * qj != 0.f;
    if (!el && !lj) return;
    const float rinv = adj_rsqrt(r2);
    if (el) {
        float ex;
        phi += qj * nb_erfc_ex(R.alpha * r2 * rinv, r2 * R.ex2c, &ex) * rinv;
    }
    if (lj) {
        const float s2 = rinv * rinv, s6 = s2 * s2 * s2;
        float a, b;
        if (!R.arith) {
            a = lji.x * ljj.x * s6 * s6;
            b = lji.y * ljj.y * s6;
        } else {
            const float aa = lji.x * ljj.x, sg = 0.5f * (lji.y + ljj.y);
            float b1 = sg * sg * sg;
            b1 = b1 * b1;
            b = aa * b1 * s6;
            a = aa * b1 * b1 * s6 * s6;
        }
        const float g = 6.f * a - 3.f * b;
        de += (a - b) * inv2e_i;
        if (!R.arith) {
            if (sig_i > 0.f) ds += g / sig_i;
        } else {
            float ej, sj;
            lj_decode_f(1, ljj.x, ljj.y, ej, sj);
            const float sij = 0.5f * (sig_i + sj);
            if (sij > 0.f) ds += g / sij;
        }
    }
}

// water molecule per thread (FP32 pairs): W1 (nine site pairs per molecule pair, O-O LJ) and W2
template <typename E>
__global__ void __launch_bounds__(128) k_adj_water_f(int nW, const RepDev *__restrict__ reps,
                                                     const int *__restrict__ site_rep,
                                                     const int *__restrict__ site_orig,
                                                     const float4 *__restrict__ pos, const float4 *__restrict__ woff,
                                                     const float2 *__restrict__ lj,
                                                     const unsigned *__restrict__ sflags,
                                                     const int2 *__restrict__ wl1_cnt, const void *__restrict__ wl1,
                                                     int cap_row, const int *__restrict__ wl2_off,
                                                     const int *__restrict__ wl2, int cap2, double *__restrict__ dq,
                                                     double *__restrict__ de, double *__restrict__ ds)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nW) return;
    const RepDev &R = reps[site_rep[3 * i]];
    const float4 oi = woff[3 * i];
    const float4 h1 = woff[3 * i + 1], h2 = woff[3 * i + 2];
    const float hi[3][3] = {{0.f, 0.f, 0.f}, {h1.x, h1.y, h1.z}, {h2.x, h2.y, h2.z}};
    double phi[3] = {0, 0, 0}, dE[3] = {0, 0, 0}, dS[3] = {0, 0, 0};
    float p[3] = {0.f, 0.f, 0.f}, e3[3] = {0.f, 0.f, 0.f}, s3[3] = {0.f, 0.f, 0.f};
    auto flush = [&]() {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            phi[a] += (double)p[a]; dE[a] += (double)e3[a]; dS[a] += (double)s3[a];
            p[a] = 0.f; e3[a] = 0.f; s3[a] = 0.f;
        }
    };
    float epsO, sigO;
    const float2 ljO = lj[3 * i];
    lj_decode_f(R.arith, ljO.x, ljO.y, epsO, sigO);
    const float inv2eO = epsO > 0.f ? 0.5f / epsO : 0.f, invsO = sigO > 0.f ? 1.f / sigO : 0.f;
    const float alpha = R.alpha, ex2c = R.ex2c, rmax2 = R.rmax2, rv2 = R.rv2, w12 = R.w12, w6 = R.w6;
    const int2 c = wl1_cnt[i];
    const int nn = min(c.x, cap_row), n = min(c.x + c.y, cap_row);
    const E *row = (const E *)wl1 + (size_t)i * cap_row;
    const int base = sizeof(E) == 2 ? R.wat0 : 0;   // uint16 entries: offsets from the replica's first water
    int cnt = 0;
    for (int v = 0; v < n; ++v) {
        nb_prefetch_l1(row + min(v + 32, n - 1));
        const int j = base + (int)row[v < nn ? v : cap_row - 1 - (v - nn)];
        const float4 oj = woff[3 * j];
        float dx = oi.x - oj.x, dy = oi.y - oj.y, dz = oi.z - oj.z;
        dx = nb_shift(R, 0, dx, rintf(dx * R.invL[0]));
        dy = nb_shift(R, 1, dy, rintf(dy * R.invL[1]));
        dz = nb_shift(R, 2, dz, rintf(dz * R.invL[2]));
        const float r2oo = dx * dx + dy * dy + dz * dz;
        if (r2oo > rmax2) continue;
        const float4 j1 = woff[3 * j + 1], j2 = woff[3 * j + 2];
        const float hj[3][3] = {{0.f, 0.f, 0.f}, {j1.x, j1.y, j1.z}, {j2.x, j2.y, j2.z}};
        const float qj[3] = {oj.w, pos[3 * j + 1].w, pos[3 * j + 2].w};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const float ex = hi[a][0] + dx - hj[b][0], ey = hi[a][1] + dy - hj[b][1], ez = hi[a][2] + dz - hj[b][2];
                const float r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                const float rinv = adj_rsqrt(r2);
                float exv;
                p[a] += qj[b] * nb_erfc_ex(alpha * r2 * rinv, r2 * ex2c, &exv) * rinv;
            }
        if (r2oo <= rv2) {
            const float ri = adj_rsqrt(r2oo), s2 = ri * ri, s6 = s2 * s2 * s2;
            const float A = w12 * s6 * s6, B = w6 * s6;
            e3[0] += (A - B) * inv2eO;
            s3[0] += (6.f * A - 3.f * B) * invsO;     // sigma_ij = sigma_O for water pairs (both rules)
        }
        if (++cnt == CHUNK_ADJ) { flush(); cnt = 0; }
    }
    flush();
    cnt = 0;
    const int q0 = min(wl2_off[i], cap2), q1 = min(wl2_off[i + 1], cap2);
    float inv2e[3], sg[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float ea, sa;
        const float2 l = lj[3 * i + a];
        lj_decode_f(R.arith, l.x, l.y, ea, sa);
        inv2e[a] = ea > 0.f ? 0.5f / ea : 0.f;
        sg[a] = sa;
    }
    for (int k = q0; k < q1; ++k) {
        const int s = wl2[k];
        const float4 xj = pos[s];
        const float2 ljj = lj[s];
        const unsigned fj = sflags[s];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float4 xi = pos[3 * i + a];
            float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            dx = nb_shift(R, 0, dx, rintf(dx * R.invL[0]));
            dy = nb_shift(R, 1, dy, rintf(dy * R.invL[1]));
            dz = nb_shift(R, 2, dz, rintf(dz * R.invL[2]));
            atom_pair_adj_f(R, dx * dx + dy * dy + dz * dz, xi.w, xj.w, lj[3 * i + a], ljj, sflags[3 * i + a], fj,
                            inv2e[a], sg[a], p[a], e3[a], s3[a]);
        }
        if (++cnt == CHUNK_ADJ) { flush(); cnt = 0; }
    }
    flush();
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int o = site_orig[3 * i + a];
        dq[o] = R.epstmp * phi[a];
        de[o] = dE[a];
        ds[o] = dS[a];
    }
}

// non-water atom per thread over its X list (FP32 pairs)
__global__ void __launch_bounds__(128) k_adj_atom_f(int nA, int nW, const RepDev *__restrict__ reps,
                                                    const int *__restrict__ site_rep,
                                                    const int *__restrict__ site_orig, const float4 *__restrict__ pos,
                                                    const float2 *__restrict__ lj, const unsigned *__restrict__ sflags,
                                                    const int *__restrict__ xl_off, const int *__restrict__ xl, int capx,
                                                    double *__restrict__ dq, double *__restrict__ de,
                                                    double *__restrict__ ds)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nA) return;
    const int si = 3 * nW + k;
    const RepDev &R = reps[site_rep[si]];
    const float4 xi = pos[si];
    const float2 lji = lj[si];
    const unsigned fi = sflags[si];
    float ei, sgi;
    lj_decode_f(R.arith, lji.x, lji.y, ei, sgi);
    const float inv2e = ei > 0.f ? 0.5f / ei : 0.f;
    double phi = 0, dE = 0, dS = 0;
    float p = 0.f, e1 = 0.f, s1 = 0.f;
    int cnt = 0;
    const int q1 = min(xl_off[k + 1], capx);
    for (int q = min(xl_off[k], capx); q < q1; ++q) {
        nb_prefetch_l1(xl + min(q + 32, q1 - 1));
        const int s = xl[q];
        const float4 xj = pos[s];
        float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        dx = nb_shift(R, 0, dx, rintf(dx * R.invL[0]));
        dy = nb_shift(R, 1, dy, rintf(dy * R.invL[1]));
        dz = nb_shift(R, 2, dz, rintf(dz * R.invL[2]));
        atom_pair_adj_f(R, dx * dx + dy * dy + dz * dz, xi.w, xj.w, lji, lj[s], fi, sflags[s], inv2e, sgi, p, e1, s1);
        if (++cnt == CHUNK_ADJ) {
            phi += (double)p; dE += (double)e1; dS += (double)s1;
            p = 0.f; e1 = 0.f; s1 = 0.f; cnt = 0;
        }
    }
    phi += (double)p; dE += (double)e1; dS += (double)s1;
    const int o = site_orig[si];
    dq[o] = R.epstmp * phi;
    de[o] = dE;
    ds[o] = dS;
}

// per caller atom: exclusion erf corrections, 1-4 terms, self energy (FP64 coordinates)
__global__ void k_adj_excl14(int natom, const int *__restrict__ atom_rep, const RepDev *__restrict__ reps,
                             const double *__restrict__ coor, const double *__restrict__ q,
                             const double2 *__restrict__ lj, const int *__restrict__ ex_off,
                             const int *__restrict__ ex_j, const int *__restrict__ p_off, const int *__restrict__ p_j,
                             const double *__restrict__ p_par, double *__restrict__ dq, double *__restrict__ de,
                             double *__restrict__ ds)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natom) return;
    const RepDev &R = reps[atom_rep[a]];
    const double xa = coor[3 * (size_t)a], ya = coor[3 * (size_t)a + 1], za = coor[3 * (size_t)a + 2];
    double phi = -2.0 * R.alphad * (NB_TWO_OVER_SQRTPI * 0.5) * R.epstmp * q[a];   // self energy
    double dE = 0, dS = 0, ea, sa;
    lj_decode(R.arith, lj[a].x, lj[a].y, ea, sa);
    for (int k = ex_off[a]; k < ex_off[a + 1]; ++k) {
        const int b = ex_j[k];
        const double rx = xa - coor[3 * (size_t)b], ry = ya - coor[3 * (size_t)b + 1], rz = za - coor[3 * (size_t)b + 2];
        const double r = sqrt(rx * rx + ry * ry + rz * rz);
        phi -= R.epstmp * q[b] * erf(R.alphad * r) / r;
    }
    for (int k = p_off[a]; k < p_off[a + 1]; ++k) {
        const int b = p_j[k];
        const double *p = p_par + 3 * (size_t)k;
        const double rx = xa - coor[3 * (size_t)b], ry = ya - coor[3 * (size_t)b + 1], rz = za - coor[3 * (size_t)b + 2];
        const double s2 = 1.0 / (rx * rx + ry * ry + rz * rz), s6 = s2 * s2 * s2;
        if (p[0] > 1e-12) {
            double eb, sb;
            lj_decode(R.arith, lj[b].x, lj[b].y, eb, sb);
            lj_adj(R.arith, p[0] * s6 * s6, p[1] * s6, ea, sa, sb, dE, dS);
        }
        if (fabs(p[2]) > 1e-12 && fabs(q[a]) > 1e-12) phi += p[2] / q[a] * sqrt(s2);
    }
    dq[a] += phi;
    de[a] += dE;
    ds[a] += dS;
}

// PME: fc * sum(theta * potential grid) at each site, from the real planes k_plane_inv_f
// leaves in the grid storage (mixed path)
__global__ void k_adj_pme_f(int nsite, const int *__restrict__ site_rep, const int *__restrict__ site_orig,
                            const RepDev *__restrict__ reps, const float4 *__restrict__ fr,
                            const float2 *__restrict__ grid, double *__restrict__ dq)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    const RepDev &R = reps[site_rep[s]];
    const float4 f = fr[s];
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3;
    const size_t zs = (size_t)R.n1h * n2 * 2;
    const float *Q = (const float *)(grid + R.g0);
    int i1, i2, i3;
    float w1, w2, w3;
    pme_fr_split(f.x, i1, w1);
    pme_fr_split(f.y, i2, w2);
    pme_fr_split(f.z, i3, w3);
    double th[3][4];
    const double w[3] = {(double)w1, (double)w2, (double)w3};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = w[d], u2 = u * u, u3 = u2 * u, m = 1.0 - u;
        th[d][0] = m * m * m / 6.0;
        th[d][1] = (4.0 - 6.0 * u2 + 3.0 * u3) / 6.0;
        th[d][2] = (1.0 + 3.0 * (u + u2 - u3)) / 6.0;
        th[d][3] = u3 / 6.0;
    }
    auto wrap = [](int k, int n) { return k < 0 ? k + n : (k >= n ? k - n : k); };
    double v = 0.0;
    for (int t3 = 0; t3 < 4; ++t3) {
        const float *P = Q + wrap(i3 - 3 + t3, n3) * zs;
        for (int t2 = 0; t2 < 4; ++t2) {
            const float *row = P + wrap(i2 - 3 + t2, n2) * n1;
            double sx = 0.0;
            for (int t1 = 0; t1 < 4; ++t1) sx += th[0][t1] * (double)row[wrap(i1 - 3 + t1, n1)];
            v += sx * th[1][t2] * th[2][t3];
        }
    }
    dq[site_orig[s]] += R.fcd * v;
}

// PME on the plain path: fc * the four plane shares of the potential at each site
__global__ void k_adj_pme_d(int nsite, const int *__restrict__ site_rep, const int *__restrict__ site_orig,
                            const RepDev *__restrict__ reps, const double *__restrict__ phi4, double *__restrict__ dq)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    const double *p = phi4 + 4 * (size_t)s;
    dq[site_orig[s]] += reps[site_rep[s]].fcd * ((p[0] + p[1]) + (p[2] + p[3]));
}

template <typename T>
void adjoint_pairs(NbCtx *c, double *d_dq, double *d_de, double *d_ds)
{
    cudaStream_t s = c->stream;
    const int B = 128;
    if constexpr (sizeof(T) == 4) {
        if (c->nW > 0)
            (c->row16 ? k_adj_water_f<unsigned short> : k_adj_water_f<int>)<<<(int)((c->nW + B - 1) / B), B, 0, s>>>(
                (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, (const float4 *)c->d_pos,
                (const float4 *)c->d_woff, (const float2 *)c->d_site_lj, c->d_site_flags, c->d_wl1_cnt, c->d_wl1,
                c->cap_row1, c->d_wl2_off, c->d_wl2, cap_int(c->cap_wl2), d_dq, d_de, d_ds);
        if (c->nA > 0)
            k_adj_atom_f<<<(int)((c->nA + B - 1) / B), B, 0, s>>>(
                (int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, (const float4 *)c->d_pos,
                (const float2 *)c->d_site_lj, c->d_site_flags, c->d_xl_off, c->d_xl, cap_int(c->cap_xl), d_dq, d_de,
                d_ds);
        return;
    }
    if (c->nW > 0)
        (c->row16 ? k_adj_water<T, unsigned short> : k_adj_water<T, int>)<<<(int)((c->nW + B - 1) / B), B, 0, s>>>(
            (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, c->d_pos, c->d_woff, c->d_site_lj,
            c->d_site_flags, c->d_wl1_cnt, c->d_wl1, c->cap_row1, c->d_wl2_off, c->d_wl2, cap_int(c->cap_wl2), d_dq,
            d_de, d_ds);
    if (c->nA > 0)
        k_adj_atom<T><<<(int)((c->nA + B - 1) / B), B, 0, s>>>(
            (int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep, c->d_site_orig, c->d_pos, c->d_site_lj,
            c->d_site_flags, c->d_xl_off, c->d_xl, cap_int(c->cap_xl), d_dq, d_de, d_ds);
}

}  // namespace

void nb_launch_pme_potential(NbCtx *c, double *phi4);

int nb_adjoint(NbCtx *c, double *d_dq, double *d_de, double *d_ds)
{
    cudaStream_t s = c->stream;
    const int B = 128;
    if (c->precision == MOIL_NB_FP64) adjoint_pairs<double>(c, d_dq, d_de, d_ds);
    else adjoint_pairs<float>(c, d_dq, d_de, d_ds);
    k_adj_excl14<<<(int)((c->natom + B - 1) / B), B, 0, s>>>(
        (int)c->natom, c->d_atom_rep, c->d_reps, c->d_coor, c->d_q, c->d_lj_d, c->d_ex_off, c->d_ex_j,
        c->d_p14_off, c->d_p14_j, c->d_p14_par, d_dq, d_de, d_ds);
    if (c->precision == MOIL_NB_FP64) {
        nb_launch_pme_potential(c, c->d_adj_phi);
        k_adj_pme_d<<<(int)((c->nsite + B - 1) / B), B, 0, s>>>((int)c->nsite, c->d_site_rep, c->d_site_orig,
                                                              c->d_reps, c->d_adj_phi, d_dq);
    } else {
        k_adj_pme_f<<<(int)((c->nsite + B - 1) / B), B, 0, s>>>((int)c->nsite, c->d_site_rep, c->d_site_orig,
                                                              c->d_reps, (const float4 *)c->d_fr,
                                                              (const float2 *)c->d_grid, d_dq);
    }
    NB_CUDA_OK(c, cudaGetLastError());
    return MOIL_NB_OK;
}
