// nb_realspace.cu -- real-space LJ + erfc-Coulomb, exclusion/1-4 corrections, finalize.
//
// Pair semantics are MOIL's predicate evaluated at the current coordinates:
//   water-water   pot/watwat_ewald.f:131-612 (+ images, symm/symwat_ewald.f): the molecule
//                 pair is in iff O-O r^2 <= max(cutvdw2, cutele2); then all 9 site pairs get
//                 erfc-Coulomb with the O-O image shift and no per-site cutoff, O-O LJ if
//                 r^2 <= cutvdw2.
//   other pairs   pot/cdie_ewald.f:313-671 (+ symm/symcdie_ewald.f) with the lists of
//                 pot/nbond.f:115-149: LJ iff r^2 < cutvdw2 (and not the geometric hydrogen
//                 rule inside cutele2), Coulomb iff both charged and r^2 < max(cutvdw2, cutele2).
//   primary vs image: a pair whose minimum-image shift is zero is a primary-box pair
//                 (e_vdw/e_el); any other shift is one of MOIL's translated images
//                 (e_vsym/e_lsym).
// Lists are full (each pair appears under both atoms); every lane owns its own gradient,
// so nothing is written twice and no atomics are needed.  Energies are halved at the end.
#include "nb_internal.h"

namespace {

#define CHUNK 64

template <typename T>
__device__ __forceinline__ void lj_switch_apply(const RepDev &R, T r2, T &e1, T &df1)
{
    if (R.lj_switch && r2 > (T)R.ron2) {
        T d = (T)R.rv2 - r2;
        T sw = d * d * ((T)R.rv2 + (T)2 * r2 - (T)3 * (T)R.ron2) * (T)R.swden;
        T dsw = (T)12 * d * ((T)R.ron2 - r2) * (T)R.swden;
        df1 = df1 * sw + e1 * dsw;
        e1 *= sw;
    }
}

template <typename T> struct Consts;
template <> struct Consts<float> {
    __device__ static float qq(const RepDev &R, int k) { return R.qq[k]; }
    __device__ static float w12(const RepDev &R) { return R.w12; }
    __device__ static float w6(const RepDev &R) { return R.w6; }
    __device__ static float alpha(const RepDev &R) { return R.alpha; }
    __device__ static float epstmp(const RepDev &R) { return (float)R.epstmp; }
};
template <> struct Consts<double> {
    __device__ static double qq(const RepDev &R, int k) { return R.qqd[k]; }
    __device__ static double w12(const RepDev &R) { return R.w12d; }
    __device__ static double w6(const RepDev &R) { return R.w6d; }
    __device__ static double alpha(const RepDev &R) { return R.alphad; }
    __device__ static double epstmp(const RepDev &R) { return R.epstmp; }
};

// one non-water-type pair (cdie_ewald list1/2/3 semantics); d already minimum-imaged
// vir receives MOIL's LJ virial term of the pair, -df1 r^2 (cdie_ewald_press.f:413-419)
template <typename T>
__device__ __forceinline__ T atom_pair(const RepDev &R, T r2, T qi, T qj, T e12i, T e6i, T e12j, T e6j,
                                       unsigned fi, unsigned fj, T &eel, T &elj, T &vir, int &npair)
{
    bool hr = !R.arith && R.hvdw0 && ((fi | fj) & SF_HTINY) && r2 < (T)R.re2;
    bool lj = r2 < (T)R.rv2 && !hr;
    T qq = qi * qj;
    bool el = r2 < (T)R.rmax2 && qq != (T)0;
    if (!lj && !el) return (T)0;
    ++npair;
    T rinv = nb_rsqrt(r2);
    T s2 = rinv * rinv;
    T df = 0;
    if (el) {
        T x = Consts<T>::alpha(R) * r2 * rinv;
        T ex;
        T erfcv = nb_erfc_ex(x, r2 * (T)R.ex2c, &ex);
        qq *= Consts<T>::epstmp(R);
        T e = qq * erfcv * rinv;
        df = -(e + qq * (T)R.c2a * ex) * s2;
        eel += e;
    }
    if (lj) {
        // r^-6 and r^-12 amplify the approximate FP32 rsqrt's error 6 and 12 times: one
        // Newton step (FP32) first
        const T rl = sizeof(T) == 4 ? fma((T)-0.5 * rinv, fma(r2, s2, (T)-1), rinv) : rinv;
        s2 = rl * rl;
        T s6 = s2 * s2 * s2, A, B;
        if (!R.arith) {
            A = e12i * e12j * s6 * s6;
            B = e6i * e6j * s6;
        } else {
            T aa = e12i * e12j, sg = (T)0.5 * (e6i + e6j);
            T b1 = sg * sg * sg;
            b1 = b1 * b1;
            B = aa * b1 * s6;
            A = aa * b1 * b1 * s6 * s6;
        }
        T e1 = A - B;
        T df1 = (T)-6 * s2 * (A + e1);
        lj_switch_apply<T>(R, r2, e1, df1);
        elj += e1;
        vir -= df1 * r2;
        df += df1;
    }
    return df;
}

template <typename T>
__device__ __forceinline__ void min_image(const RepDev &R, T &dx, T &dy, T &dz, bool &img)
{
    T nx = nb_rint(dx * rep_invL<T>(R, 0)), ny = nb_rint(dy * rep_invL<T>(R, 1)), nz = nb_rint(dz * rep_invL<T>(R, 2));
    dx = nb_shift(R, 0, dx, nx);
    dy = nb_shift(R, 1, dy, ny);
    dz = nb_shift(R, 2, dz, nz);
    img = (nx != (T)0) | (ny != (T)0) | (nz != (T)0);
}

__device__ __forceinline__ void flush(float g[], long long G[], int n)
{
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (k < n) { G[k] += nb_fix(g[k]); g[k] = 0.f; }
    }
}
__device__ __forceinline__ void flush(double g[], long long G[], int n)
{
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (k < n) { G[k] += nb_fix(g[k]); g[k] = 0.0; }
    }
}

// water sites of molecule i against its W2 list of non-water atoms: atom semantics per site
// pair; partial gradients and energies go to g / e4, flushed every CHUNK entries
template <typename T, typename Flush>
__device__ __forceinline__ void water_vs_atoms(const RepDev &R, int i, const typename vec4<T>::type *pos,
                                               const void *lj_v, const unsigned *__restrict__ sflags,
                                               const int *__restrict__ wl2_off, const int *__restrict__ wl2, int cap2,
                                               T g[9], T e4[4], int &npair, Flush &flush_all)
{
    typedef typename vec4<T>::type T4;
    typedef typename cplx<T>::type T2;
    // an overflowed list (offsets past the capacity) is read within the buffer; the
    // evaluation reports the overflow and is redone with a larger one
    const int q0 = min(wl2_off[i], cap2), q1 = min(wl2_off[i + 1], cap2);
    if (q0 >= q1) return;
    const T2 *lj = (const T2 *)lj_v;
    const T4 si[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    const T2 lji[3] = {lj[3 * i], lj[3 * i + 1], lj[3 * i + 2]};
    const unsigned fi[3] = {sflags[3 * i], sflags[3 * i + 1], sflags[3 * i + 2]};
    int cnt = 0;
    for (int k = q0; k < q1; ++k) {
        nb_prefetch_l1(wl2 + min(k + 32, q1 - 1));
        int s = wl2[k];
        T4 xj = pos[s];
        T2 ljj = lj[s];
        unsigned fj = sflags[s];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            T dx = si[a].x - xj.x, dy = si[a].y - xj.y, dz = si[a].z - xj.z;
            bool img;
            min_image<T>(R, dx, dy, dz, img);
            T r2 = dx * dx + dy * dy + dz * dz;
            T eel = 0, elj = 0, vir = 0;   // the virial of these pairs is counted by k_atom
            T df = atom_pair<T>(R, r2, si[a].w, xj.w, lji[a].x, lji[a].y, ljj.x, ljj.y, fi[a], fj, eel, elj, vir,
                                npair);
            g[3 * a] += df * dx;
            g[3 * a + 1] += df * dy;
            g[3 * a + 2] += df * dz;
            e4[img ? 1 : 0] += elj;
            e4[img ? 3 : 2] += eel;
        }
        if (++cnt == CHUNK) { flush_all(); cnt = 0; }
    }
    flush_all();
}

// ---------------------------------------------------------------------------------
// water molecule per thread: W1 (water-water, 9 site pairs) then W2 (water-site x other).
// Per-lane FP32 partial gradients and energies are flushed every CHUNK list entries into
// int64 / FP64 accumulators kept in shared memory (one column per thread), which keeps
// them out of the register file.
#define WBLOCK 128

// water i's W1 row: entry v is the v-th in-cutoff molecule from the front for v < nn, then
// the skin-only molecules from the back of the row
template <typename E>
struct W1Row {
    const E *row;
    int nn, n, cap, base;
    __device__ W1Row(const int2 *__restrict__ cnt, const void *wl1, int cap_row, int i, int base_)
    {
        const int2 c = cnt[i];
        row = (const E *)wl1 + (size_t)i * cap_row;
        // an overflowed row (counts above the capacity) is read within the row; the
        // evaluation reports the overflow and is redone with larger rows
        nn = min(c.x, cap_row);
        n = min(c.x + c.y, cap_row);
        cap = cap_row;
        base = sizeof(E) == 2 ? base_ : 0;     // uint16 entries are offsets from the replica's first water
    }
    __device__ const E *addr(int v) const { return row + (v < nn ? v : cap - 1 - (v - nn)); }
    __device__ int at(int v) const { return base + (int)*addr(v); }
};

// Plain FP64 path: one water per thread in blocks of WBLOCK64 (the FP64 pipe of this GPU is a
// small fraction of the FP32 one, so a replica of a few hundred waters needs every
// multiprocessor it can get: 32-thread blocks spread it over four times more SMs than 128)
#define WBLOCK64 32
template <typename T, typename E>
__global__ void __launch_bounds__(WBLOCK64) k_water(int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                                                     const void *pos_v, const void *woff_v, const void *lj_v,
                                                     const unsigned *__restrict__ sflags,
                                                     const int2 *__restrict__ wl1_cnt, const void *__restrict__ wl1,
                                                     int cap_row, const int *__restrict__ wl2_off,
                                                     const int *__restrict__ wl2, int cap2, long long *__restrict__ grad,
                                                     double *__restrict__ e_unit)
{
    __shared__ long long sG[9][WBLOCK64];
    __shared__ double sE[6][WBLOCK64];
    const int t = threadIdx.x;
    int i = blockIdx.x * WBLOCK64 + t;
    if (i >= nW) return;
    typedef typename vec4<T>::type T4;
    typedef typename cplx<T>::type T2;
    const T4 *pos = (const T4 *)pos_v;
    const T4 *woff = (const T4 *)woff_v;
    const RepDev &R = reps[site_rep[3 * i]];
#pragma unroll
    for (int k = 0; k < 9; ++k) sG[k][t] = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) sE[k][t] = 0.0;
    const T4 oi0 = pos[3 * i];
    // i-site offsets from O (a = 0 is O itself)
    const T4 oi1 = woff[3 * i + 1], oi2 = woff[3 * i + 2];
    const T oi[3][3] = {{(T)0, (T)0, (T)0}, {oi1.x, oi1.y, oi1.z}, {oi2.x, oi2.y, oi2.z}};
    T g[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = 0;
    T e4[6] = {0, 0, 0, 0, 0, 0};   // LJ prim, LJ img, Coulomb prim, Coulomb img, LJ virial prim, img
    auto flush_all = [&]() {
#pragma unroll
        for (int k = 0; k < 9; ++k) { sG[k][t] += nb_fix(g[k]); g[k] = 0; }
#pragma unroll
        for (int k = 0; k < 6; ++k) { sE[k][t] += (double)e4[k]; e4[k] = 0; }
    };
    int npair = 0;
    const T iL0 = rep_invL<T>(R, 0), iL1 = rep_invL<T>(R, 1), iL2 = rep_invL<T>(R, 2);
    const T rmax2 = (T)R.rmax2, rv2 = (T)R.rv2, alpha = Consts<T>::alpha(R), ex2c = (T)R.ex2c, c2a = (T)R.c2a;
    const T qOO = Consts<T>::qq(R, 0), qOH = Consts<T>::qq(R, 1), qHH = Consts<T>::qq(R, 2);
    const T w12 = Consts<T>::w12(R), w6 = Consts<T>::w6(R);
    const W1Row<E> L1(wl1_cnt, wl1, cap_row, i, R.wat0);
    int cnt = 0;
    // software pipeline: the next entry's index and oxygen are loaded one iteration ahead
    int jn = L1.n > 0 ? L1.at(0) : 0;
    T4 ojn = pos[3 * jn];
    for (int k = 0; k < L1.n; ++k) {
        const int j = jn;
        const T4 oj = ojn;
        if (k + 1 < L1.n) {
            jn = L1.at(k + 1);
            ojn = pos[3 * jn];
        }
        T dx = oi0.x - oj.x, dy = oi0.y - oj.y, dz = oi0.z - oj.z;
        T nx = nb_rint(dx * iL0), ny = nb_rint(dy * iL1), nz = nb_rint(dz * iL2);
        dx = nb_shift(R, 0, dx, nx);
        dy = nb_shift(R, 1, dy, ny);
        dz = nb_shift(R, 2, dz, nz);
        T r2oo = dx * dx + dy * dy + dz * dz;
        if (r2oo <= rmax2) {
            T4 oj1 = woff[3 * j + 1], oj2 = woff[3 * j + 2];
            // q[b] = (O_i - O_j - nL) - offset_j[b]; site displacement = offset_i[a] + q[b]
            const T q[3][3] = {{dx, dy, dz}, {dx - oj1.x, dy - oj1.y, dz - oj1.z}, {dx - oj2.x, dy - oj2.y, dz - oj2.z}};
            T e_el = 0, e_lj = 0, v_lj = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    T ddx = a ? oi[a][0] + q[b][0] : q[b][0];
                    T ddy = a ? oi[a][1] + q[b][1] : q[b][1];
                    T ddz = a ? oi[a][2] + q[b][2] : q[b][2];
                    T rr2 = ddx * ddx + ddy * ddy + ddz * ddz;
                    T rinv = nb_rsqrt(rr2);
                    T s2 = rinv * rinv;
                    T x = alpha * rr2 * rinv;
                    T ex;
                    T erfcv = nb_erfc_ex(x, rr2 * ex2c, &ex);
                    const T qq = (a == 0 && b == 0) ? qOO : ((a == 0 || b == 0) ? qOH : qHH);
                    T e = qq * erfcv * rinv;
                    T df = -(e + qq * c2a * ex) * s2;
                    if (a == 0 && b == 0) {
                        if (rr2 <= rv2) {
                            T s6 = s2 * s2 * s2, A = w12 * s6 * s6, B = w6 * s6;
                            T e1 = A - B, df1 = (T)-6 * s2 * (A + e1);
                            lj_switch_apply<T>(R, rr2, e1, df1);
                            e_lj += e1;
                            v_lj -= df1 * rr2;   // watwat_ewald_press.f:146-152
                            df += df1;
                        }
                    }
                    e_el += e;
                    g[3 * a] += df * ddx;
                    g[3 * a + 1] += df * ddy;
                    g[3 * a + 2] += df * ddz;
                }
            }
            const bool img = (nx != (T)0) | (ny != (T)0) | (nz != (T)0);
            e4[img ? 1 : 0] += e_lj;
            e4[img ? 3 : 2] += e_el;
            e4[img ? 5 : 4] += v_lj;
            npair += 9;
        }
        if (++cnt == CHUNK) { flush_all(); cnt = 0; }
    }
    flush_all();
    water_vs_atoms<T>(R, i, pos, lj_v, sflags, wl2_off, wl2, cap2, g, e4, npair, flush_all);
#pragma unroll
    for (int k = 0; k < 9; ++k) grad[(size_t)9 * i + k] = sG[k][t];
    double *eu = e_unit + NB_EU * (size_t)i;
    eu[0] = sE[0][t]; eu[1] = sE[1][t]; eu[2] = sE[2][t]; eu[3] = sE[3][t]; eu[4] = (double)npair;
    eu[5] = 0.0; eu[6] = sE[4][t]; eu[7] = sE[5][t];
}

// FP32 water exclusion corrections (cdie_ewald.f:117-199 for the pairs O-H1, O-H2, H1-H2 of
// one rigid water): the three intramolecular displacements come from the FP64-formed H
// offsets h1, h2, so no absolute FP32 coordinate enters; erf(x)/x from its Taylor series in
// u = x^2 (9 terms, truncation below 6e-9 for u <= 0.5), erff beyond.  Adds the gradient of
// the three sites to g[3 * site + axis] and returns the energy.  With R.wref the returned
// energy is the difference from the replica's reference water (wcorr0, added in FP64 by the
// energy reduction): coef * (r^2 - t0) * Q(r^2) per pair, Q the quotient of the series by
// (r^2 - t0), which keeps the FP32 error a fraction of a small difference.
__device__ __forceinline__ float water_intra_f(const RepDev &R, float4 h1, float4 h2, const float q[3], float g[9])
{
    // displacement x_a - x_b for the pairs (O,H1), (O,H2), (H1,H2)
    const float d[3][3] = {{-h1.x, -h1.y, -h1.z}, {-h2.x, -h2.y, -h2.z}, {h1.x - h2.x, h1.y - h2.y, h1.z - h2.z}};
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    const float al = R.alpha, ke = (float)R.epstmp, c2 = (float)NB_TWO_OVER_SQRTPI;
    float ecorr = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float rx = d[k][0], ry = d[k][1], rz = d[k][2];
        const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz)), u = al * al * r2;
        const float qq = q[pa[k]] * q[pb[k]] * ke;
        float e = 0.f, df;
        if (u <= 0.5f) {
            float ds = 8.f / 685440.f;
            ds = fmaf(ds, u, -7.f / 75600.f); ds = fmaf(ds, u, 6.f / 9360.f); ds = fmaf(ds, u, -5.f / 1320.f);
            ds = fmaf(ds, u, 4.f / 216.f); ds = fmaf(ds, u, -3.f / 42.f); ds = fmaf(ds, u, 0.2f);
            ds = fmaf(ds, u, -1.f / 3.f);
            if (!R.wref) {
                float s = 1.f / 685440.f;
                s = fmaf(s, u, -1.f / 75600.f); s = fmaf(s, u, 1.f / 9360.f); s = fmaf(s, u, -1.f / 1320.f);
                s = fmaf(s, u, 1.f / 216.f); s = fmaf(s, u, -1.f / 42.f); s = fmaf(s, u, 0.1f);
                s = fmaf(s, u, -1.f / 3.f); s = fmaf(s, u, 1.f);
                e = -qq * al * c2 * s;
            }
            df = -qq * 2.f * al * al * al * c2 * ds;
        } else {
            const float rij = sqrtf(r2), sinv = 1.f / rij, x = al * rij;
            const float erfv = erff(x), derfc = c2 * expf(-x * x);
            if (!R.wref) e = -qq * sinv * erfv;
            df = qq * sinv * (sinv * sinv * erfv - sinv * al * derfc);
        }
        if (R.wref) {
            const int ty = k == 2 ? 1 : 0;    // O-H, O-H, H-H
            float qv = R.wq[ty][7];
#pragma unroll
            for (int m = 6; m >= 0; --m) qv = fmaf(qv, r2, R.wq[ty][m]);
            e = R.wcoef[ty] * ((r2 - R.wt0[ty]) * qv);
        }
        ecorr += e;
        const int a = pa[k], b = pb[k];
        g[3 * a] += df * rx; g[3 * a + 1] += df * ry; g[3 * a + 2] += df * rz;
        g[3 * b] -= df * rx; g[3 * b + 1] -= df * ry; g[3 * b + 2] -= df * rz;
    }
    return ecorr;
}

// ---------------------------------------------------------------------------------
// FP32 water kernel on the packed two-lane FP32 pipe: list entries are taken two at a
// time and every quantity of the 9 site pairs is a float2 over (entry k, entry k+1).  A
// molecule outside the O-O cutoff (or the missing partner of an odd tail) is moved 1e4 Å
// away, where erfc and exp underflow to exactly zero, so it adds nothing without a branch.
// Gradients are accumulated per lane as float2 and folded at each flush; W2 (water sites vs
// non-water atoms) runs the scalar code of k_water.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// VIR: also the water-water LJ virial terms (two more accumulators, which the 128-register
// budget of the plain evaluation does not hold without spilling; off unless requested)
template <bool VIR, typename E>
__global__ void __launch_bounds__(WBLOCK, 4) k_water_f(int nW, const RepDev *__restrict__ reps,
                                                       const int *__restrict__ site_rep, const float4 *__restrict__ pos,
                                                       const float4 *__restrict__ woff, const void *lj_v,
                                                       const unsigned *__restrict__ sflags,
                                                       const int2 *__restrict__ wl1_cnt, const void *__restrict__ wl1,
                                                       int cap_row, const int *__restrict__ wl2_off,
                                                       const int *__restrict__ wl2, int cap2, long long *__restrict__ grad,
                                                       double *__restrict__ e_unit, int intra)
{
    __shared__ long long sG[9][WBLOCK];
    __shared__ float2 sE[6][WBLOCK];     // energies as unevaluated sums hi + lo (no FP64 pipe)
    const int t = threadIdx.x;
    const int i = blockIdx.x * WBLOCK + t;
    if (i >= nW) return;
    const RepDev &R = reps[site_rep[3 * i]];
#pragma unroll
    for (int k = 0; k < 9; ++k) sG[k][t] = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) sE[k][t] = make_float2(0.f, 0.f);
    const float4 oi0 = woff[3 * i];
    const float4 oi1 = woff[3 * i + 1], oi2 = woff[3 * i + 2];
    // H offsets of molecule i, duplicated into both lanes
    const float2 hi[2][3] = {{f2(oi1.x), f2(oi1.y), f2(oi1.z)}, {f2(oi2.x), f2(oi2.y), f2(oi2.z)}};
    float2 G[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) G[k] = f2(0.f);
    float g[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = 0.f;
    // LJ prim, LJ img, Coulomb prim, Coulomb img (, LJ virial prim, LJ virial img)
    constexpr int NE = VIR ? 6 : 4;
    float e4[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) e4[k] = 0.f;
    // the molecule's own exclusion corrections (every water excludes exactly its three pairs)
    float ecorr = 0.f;
    if (intra) {
        const float qs[3] = {oi0.w, pos[3 * i + 1].w, pos[3 * i + 2].w};
        ecorr = water_intra_f(R, oi1, oi2, qs, g);
    }
    auto flush_all = [&]() {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            sG[k][t] += nb_fix(g[k] - (G[k].x + G[k].y));   // G holds minus the gradient
            g[k] = 0.f;
            G[k] = f2(0.f);
        }
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            // TwoSum (Knuth): hi + e4 = s + err exactly; the errors collect in lo
            const float2 a = sE[k][t];
            const float sm = a.x + e4[k], bb = sm - a.x, err = (a.x - (sm - bb)) + (e4[k] - bb);
            sE[k][t] = make_float2(sm, a.y + err);
            e4[k] = 0.f;
        }
    };
    int npair = 0;
    const float iL0 = R.invL[0], iL1 = R.invL[1], iL2 = R.invL[2];
    const float rmax2 = R.rmax2, rv2 = R.rv2;
    const float2 palpha = f2(ERFCX_P * R.alpha), ex2c = f2(R.ex2c);
    const float2 w12 = f2(R.w12), nw6 = f2(-R.w6);
    const float2 c12 = f2(R.w12c), c6 = f2(R.w6c);
    const float qqv[3] = {R.qq[0], R.qq[1], R.qq[2]};
    const float c2a = R.c2a;
    const W1Row<E> L1(wl1_cnt, wl1, cap_row, i, R.wat0);
    const int k1 = L1.n;
    int cnt = 0;
    // next pair of entries, loaded one iteration ahead
    int ja = k1 > 0 ? L1.at(0) : 0;
    int jb = k1 > 1 ? L1.at(1) : ja;
    float4 oa = woff[3 * ja], ob = woff[3 * jb];
    for (int k = 0; k < k1; k += 2) {
        const bool hasb = k + 1 < k1;
        const int j0 = ja, j1 = jb;
        const float4 o0 = oa, o1 = ob;
        // each lane streams its own row (a DRAM stream): pull the line 32 entries ahead
        nb_prefetch_l1(L1.addr(min(k + 32, k1 - 1)));
        if (k + 2 < k1) {
            ja = L1.at(k + 2);
            jb = k + 3 < k1 ? L1.at(k + 3) : ja;
            oa = woff[3 * ja];
            ob = woff[3 * jb];
        }
        // O-O minimum image per entry; (x + 1.5*2^23) - 1.5*2^23 rounds x to nearest (|x| < 2^22)
        float dx0 = oi0.x - o0.x, dy0 = oi0.y - o0.y, dz0 = oi0.z - o0.z;
        float dx1 = oi0.x - o1.x, dy1 = oi0.y - o1.y, dz1 = oi0.z - o1.z;
        const float nx0 = fmaf(dx0, iL0, 12582912.f) - 12582912.f, ny0 = fmaf(dy0, iL1, 12582912.f) - 12582912.f, nz0 = fmaf(dz0, iL2, 12582912.f) - 12582912.f;
        const float nx1 = fmaf(dx1, iL0, 12582912.f) - 12582912.f, ny1 = fmaf(dy1, iL1, 12582912.f) - 12582912.f, nz1 = fmaf(dz1, iL2, 12582912.f) - 12582912.f;
        dx0 = nb_shift(R, 0, dx0, nx0); dy0 = nb_shift(R, 1, dy0, ny0); dz0 = nb_shift(R, 2, dz0, nz0);
        dx1 = nb_shift(R, 0, dx1, nx1); dy1 = nb_shift(R, 1, dy1, ny1); dz1 = nb_shift(R, 2, dz1, nz1);
        const float r0 = dx0 * dx0 + dy0 * dy0 + dz0 * dz0, r1 = dx1 * dx1 + dy1 * dy1 + dz1 * dz1;
        const bool in0 = r0 <= rmax2, in1 = hasb && r1 <= rmax2;
        if (in0 || in1) {
            const float4 a1 = woff[3 * j0 + 1], a2 = woff[3 * j0 + 2];
            const float4 b1 = woff[3 * j1 + 1], b2 = woff[3 * j1 + 2];
            if (!in0) { dx0 = 1.0e4f; dy0 = 0.f; dz0 = 0.f; }
            if (!in1) { dx1 = 1.0e4f; dy1 = 0.f; dz1 = 0.f; }
            // q[b] = (O_i - O_j - nL) - offset_j[b]; site displacement = offset_i[a] + q[b]
            float2 eel = f2(0.f), elj = f2(0.f), vlj = f2(0.f);
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                float2 q[3];
                if (b == 0) {
                    q[0] = f2(dx0, dx1); q[1] = f2(dy0, dy1); q[2] = f2(dz0, dz1);
                } else if (b == 1) {
                    q[0] = f2(dx0 - a1.x, dx1 - b1.x); q[1] = f2(dy0 - a1.y, dy1 - b1.y);
                    q[2] = f2(dz0 - a1.z, dz1 - b1.z);
                } else {
                    q[0] = f2(dx0 - a2.x, dx1 - b2.x); q[1] = f2(dy0 - a2.y, dy1 - b2.y);
                    q[2] = f2(dz0 - a2.z, dz1 - b2.z);
                }
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float2 ddx = a ? __fadd2_rn(hi[a - 1][0], q[0]) : q[0];
                    const float2 ddy = a ? __fadd2_rn(hi[a - 1][1], q[1]) : q[1];
                    const float2 ddz = a ? __fadd2_rn(hi[a - 1][2], q[2]) : q[2];
                    const float2 rr2 = __ffma2_rn(ddx, ddx, __ffma2_rn(ddy, ddy, __fmul2_rn(ddz, ddz)));
                    const float2 rinv = f2(nb_rsqrt_approx(rr2.x), nb_rsqrt_approx(rr2.y));
                    const float2 s2 = __fmul2_rn(rinv, rinv);
                    const float2 arg = __fmul2_rn(rr2, ex2c);
                    // erfc(x) = exp(-x^2) * t * P(A t + B), t = 1 / (1 + P x), x = alpha r, with
                    // no clamp to the fitted range x <= 4.5: beyond it the fit extrapolates
                    // smoothly (relative error 1e-5 at x = 7, 2e-3 at x = 3500, the parked
                    // entries) and exp(-x^2) < 1e-8 makes the term negligible
                    const float2 den = __ffma2_rn(palpha, __fmul2_rn(rr2, rinv), f2(1.f));
                    const float2 tt = f2(nb_rcp_approx(den.x), nb_rcp_approx(den.y));
                    const float2 u = __ffma2_rn(f2(ERFCX_A), tt, f2(ERFCX_B));
                    const float C[ERFCX_NC] = ERFCX_COEFS;
                    float2 p = f2(C[ERFCX_NC - 1]);
#pragma unroll
                    for (int m = ERFCX_NC - 2; m >= 0; --m) p = __ffma2_rn(p, u, f2(C[m]));
                    const float2 ex = f2(nb_ex2_approx(-arg.x), nb_ex2_approx(-arg.y));
                    const float2 erfcv = __fmul2_rn(ex, __fmul2_rn(tt, p));
                    const float qq = (a == 0 && b == 0) ? qqv[0] : ((a == 0 || b == 0) ? qqv[1] : qqv[2]);
                    const float2 e = __fmul2_rn(__fmul2_rn(f2(qq), erfcv), rinv);
                    // minus dE/dr / r
                    float2 mdf = __fmul2_rn(__ffma2_rn(f2(qq * c2a), ex, e), s2);
                    if (a == 0 && b == 0) {
                        // LJ powers from a Newton-refined 1/r (r^-12 amplifies rsqrt's error 12 times)
                        // rinv - rinv (r^2 rinv^2 - 1) / 2: the correction is formed as a small
                        // number, so the result keeps round-to-nearest's lack of bias
                        const float2 ri = __ffma2_rn(__fmul2_rn(f2(-0.5f), rinv), __ffma2_rn(rr2, s2, f2(-1.f)), rinv);
                        const float2 sl = __fmul2_rn(ri, ri);
                        const float2 s6 = __fmul2_rn(__fmul2_rn(sl, sl), sl);
                        const float2 A = __fmul2_rn(__fmul2_rn(w12, s6), s6);
                        // energy A (1 + c12) - B (1 + c6): c12, c6 restore the FP32 rounding of the
                        // coefficients, whose relative error would otherwise bias every pair alike
                        // (the force keeps A and B)
                        float2 e1 = __ffma2_rn(nw6, __ffma2_rn(s6, c6, s6), __ffma2_rn(A, c12, A));
                        // -df1 = 6 s2 (2A - B)
                        float2 m1 = __fmul2_rn(__fmul2_rn(f2(6.f), sl), __ffma2_rn(nw6, s6, __fadd2_rn(A, A)));
                        if (R.lj_switch) {
                            float d0 = -m1.x, d1 = -m1.y;
                            lj_switch_apply<float>(R, rr2.x, e1.x, d0);
                            lj_switch_apply<float>(R, rr2.y, e1.y, d1);
                            m1 = f2(-d0, -d1);
                        }
                        const bool l0 = rr2.x <= rv2, l1 = rr2.y <= rv2;
                        e1 = f2(l0 ? e1.x : 0.f, l1 ? e1.y : 0.f);
                        m1 = f2(l0 ? m1.x : 0.f, l1 ? m1.y : 0.f);
                        elj = __fadd2_rn(elj, e1);
                        if (VIR) vlj = __fmul2_rn(m1, rr2);   // -df1 r^2 (watwat_ewald_press.f:146-152)
                        mdf = __fadd2_rn(mdf, m1);
                    }
                    eel = __fadd2_rn(eel, e);
                    G[3 * a] = __ffma2_rn(mdf, ddx, G[3 * a]);
                    G[3 * a + 1] = __ffma2_rn(mdf, ddy, G[3 * a + 1]);
                    G[3 * a + 2] = __ffma2_rn(mdf, ddz, G[3 * a + 2]);
                }
            }
            const bool img0 = (nx0 != 0.f) | (ny0 != 0.f) | (nz0 != 0.f);
            const bool img1 = (nx1 != 0.f) | (ny1 != 0.f) | (nz1 != 0.f);
            e4[img0 ? 1 : 0] += elj.x;
            e4[img0 ? 3 : 2] += eel.x;
            if (VIR) e4[img0 ? NE - 1 : NE - 2] += vlj.x;
            e4[img1 ? 1 : 0] += elj.y;
            e4[img1 ? 3 : 2] += eel.y;
            if (VIR) e4[img1 ? NE - 1 : NE - 2] += vlj.y;
            npair += 9 * ((int)in0 + (int)in1);
        }
        cnt += 2;
        if (cnt >= CHUNK) { flush_all(); cnt = 0; }
    }
    flush_all();
    water_vs_atoms<float>(R, i, pos, lj_v, sflags, wl2_off, wl2, cap2, g, e4, npair, flush_all);
#pragma unroll
    for (int k = 0; k < 9; ++k) grad[(size_t)9 * i + k] = sG[k][t];
    double *eu = e_unit + NB_EU * (size_t)i;
#pragma unroll
    for (int k = 0; k < 4; ++k) eu[k] = (double)sE[k][t].x + (double)sE[k][t].y;
    eu[4] = (double)npair;
    eu[5] = (double)ecorr;
    eu[6] = VIR ? (double)sE[4][t].x + (double)sE[4][t].y : 0.0;
    eu[7] = VIR ? (double)sE[5][t].x + (double)sE[5][t].y : 0.0;
}

// ---------------------------------------------------------------------------------
// FP32 water kernel over half lists (k_whalf): every water-water pair is evaluated once, by
// its owner, with the pair arithmetic of k_water_f.  The owner keeps its own gradient as in
// k_water_f; the partner's side of each pair (per partner site, summed over the owner's three
// sites) goes to an int32 accumulator in shared memory indexed by the partner's place in the
// block's j-set, at 2^S units per kcal/mol/Å (S = 24 - log2 HB: HB contributions below
// NB_HALF_CAP in magnitude fit); larger contributions go directly to the int64 gradient.
// At the end the block adds its j-set sums and its own waters' gradients to the int64 site
// gradient with atomics (integer sums: the result does not depend on their order).  The
// site gradient of the waters is cleared before the launch.  Water-water energies and pair
// counts are doubled, as the energy reduction halves the full-list sums.
template <int HB> struct HalfScale;
template <> struct HalfScale<128> { static constexpr int S = 17; };
template <> struct HalfScale<256> { static constexpr int S = 16; };
template <> struct HalfScale<512> { static constexpr int S = 15; };

// VIR: also the water-water LJ virial terms (as k_water_f<true>)
template <int HB, bool VIR>
__global__ void __launch_bounds__(HB, 512 / HB) k_water_h(const int2 *__restrict__ blocks, const RepDev *__restrict__ reps,
                                                          const float4 *__restrict__ pos, const float4 *__restrict__ woff,
                                                          const void *lj_v, const unsigned *__restrict__ sflags,
                                                          const unsigned *__restrict__ hrow, int caph,
                                                          const int2 *__restrict__ hcnt, const int *__restrict__ jset,
                                                          const int *__restrict__ jn, int jcap,
                                                          const int *__restrict__ wl2_off, const int *__restrict__ wl2,
                                                          int cap2, long long *__restrict__ grad,
                                                          double *__restrict__ e_unit, int intra)
{
    constexpr int S = HalfScale<HB>::S;
    constexpr float SC = (float)(1 << S);
    constexpr int NE = VIR ? 6 : 4;
    __shared__ float2 sE[NE][HB];
    extern __shared__ int sJ[];      // [9][jcap]: partner-site gradients, 2^S units
    const int t = threadIdx.x, b = blockIdx.x;
    const int2 w = blocks[b];
    const RepDev &R = reps[w.x];
    const int nJ = jn[b];
    for (int k = t; k < nJ; k += HB)
#pragma unroll
        for (int c = 0; c < 9; ++c) sJ[c * jcap + k] = 0;
#pragma unroll
    for (int k = 0; k < NE; ++k) sE[k][t] = make_float2(0.f, 0.f);
    __syncthreads();
    const int i = w.y + t;
    if (i - R.wat0 < R.nwat) {
        const float4 oi0 = woff[3 * i];
        const float4 oi1 = woff[3 * i + 1], oi2 = woff[3 * i + 2];
        const float2 hi[2][3] = {{f2(oi1.x), f2(oi1.y), f2(oi1.z)}, {f2(oi2.x), f2(oi2.y), f2(oi2.z)}};
        float2 G[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) G[k] = f2(0.f);
        // the owner's gradient goes to the int64 site gradient with one atomic per component
        // and flush (no shared-memory slots: they would take the L1 that the gathers use)
        unsigned long long *gi = (unsigned long long *)(grad + 9 * (size_t)i);
        float g[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) g[k] = 0.f;
        // LJ prim, LJ img, Coulomb prim, Coulomb img (, LJ virial prim, LJ virial img)
        float e4[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) e4[k] = 0.f;
        double *eu = e_unit + NB_EU * (size_t)i;
        {
            // the molecule's own exclusion corrections, flushed at once (fewer live registers
            // in the pair loop)
            float ecorr = 0.f;
            if (intra) {
                const float qs[3] = {oi0.w, pos[3 * i + 1].w, pos[3 * i + 2].w};
                ecorr = water_intra_f(R, oi1, oi2, qs, g);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    const long long v = nb_fix(g[k]);
                    if (v != 0) atomicAdd(gi + k, (unsigned long long)v);
                    g[k] = 0.f;
                }
            }
            eu[5] = (double)ecorr;
        }
        // ef: 2 for the water-water energies (each pair once), 1 for the W2 part (full list)
        auto flush = [&](float ef) {
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const long long v = nb_fix(g[k] - (G[k].x + G[k].y));   // G holds minus the gradient
                if (v != 0) atomicAdd(gi + k, (unsigned long long)v);
                g[k] = 0.f;
                G[k] = f2(0.f);
            }
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                const float2 a = sE[k][t];
                const float v = ef * e4[k];
                const float sm = a.x + v, bb = sm - a.x, err = (a.x - (sm - bb)) + (v - bb);
                sE[k][t] = make_float2(sm, a.y + err);
                e4[k] = 0.f;
            }
        };
        auto flush1 = [&]() { flush(1.f); };
        // partner site `site` of both entries: its gradient shares H (x: entry 0, y: entry 1).
        // A parked entry's share is exactly zero, so it is added without a test; a share at or
        // above NB_HALF_CAP (rare) takes the int64 path for that entry and component.
        auto jadd = [&](int l0, int l1, int j0, int j1, int site, const float2 H[3]) {
            bool big = false;
#pragma unroll
            for (int d = 0; d < 3; ++d) big |= (fabsf(H[d].x) >= NB_HALF_CAP) | (fabsf(H[d].y) >= NB_HALF_CAP);
            if (!big) {
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    atomicAdd(&sJ[(3 * site + d) * jcap + l0], __float2int_rn(H[d].x * SC));
                    atomicAdd(&sJ[(3 * site + d) * jcap + l1], __float2int_rn(H[d].y * SC));
                }
            } else {
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float fe[2] = {H[d].x, H[d].y};
                    const int le[2] = {l0, l1}, je[2] = {j0, j1};
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        if (fabsf(fe[q]) < NB_HALF_CAP) atomicAdd(&sJ[(3 * site + d) * jcap + le[q]], __float2int_rn(fe[q] * SC));
                        else atomicAdd((unsigned long long *)&grad[9 * (size_t)je[q] + 3 * site + d],
                                       (unsigned long long)nb_fix(fe[q]));
                    }
                }
            }
        };
        int npair = 0;
        const float iL0 = R.invL[0], iL1 = R.invL[1], iL2 = R.invL[2];
        const float rmax2 = R.rmax2, rv2 = R.rv2;
        const float2 palpha = f2(ERFCX_P * R.alpha), ex2c = f2(R.ex2c);
        const float2 w12 = f2(R.w12), nw6 = f2(-R.w6);
        const float2 c12 = f2(R.w12c), c6 = f2(R.w6c);
        const float qqv[3] = {R.qq[0], R.qq[1], R.qq[2]};
        const float c2a = R.c2a;
        const unsigned *hr = hrow + (size_t)b * caph * HB + t;
        const int k1 = hcnt[i].y, wat0 = R.wat0;
        int cnt = 0;
        // next pair of entries, loaded one iteration ahead
        unsigned ea = k1 > 0 ? hr[0] : 0u;
        unsigned eb = k1 > 1 ? hr[HB] : ea;
        float4 oa = woff[3 * (wat0 + (int)(ea & 0xffffu))], ob = woff[3 * (wat0 + (int)(eb & 0xffffu))];
        for (int k = 0; k < k1; k += 2) {
            const bool hasb = k + 1 < k1;
            const unsigned e0 = ea, e1 = eb;
            const int j0 = wat0 + (int)(e0 & 0xffffu), j1 = wat0 + (int)(e1 & 0xffffu);
            const int l0 = (int)(e0 >> 16), l1 = (int)(e1 >> 16);
            const float4 o0 = oa, o1 = ob;
            // the warp's row lines (one 128-byte line per entry) four iterations ahead (further
            // ahead, the prefetched lines take L1 from the partner records)
            nb_prefetch_l1(hr + (size_t)min(k + 8, k1 - 1) * HB);
            if (k + 2 < k1) {
                ea = hr[(size_t)(k + 2) * HB];
                eb = k + 3 < k1 ? hr[(size_t)(k + 3) * HB] : ea;
                oa = woff[3 * (wat0 + (int)(ea & 0xffffu))];
                ob = woff[3 * (wat0 + (int)(eb & 0xffffu))];
            }
            float dx0 = oi0.x - o0.x, dy0 = oi0.y - o0.y, dz0 = oi0.z - o0.z;
            float dx1 = oi0.x - o1.x, dy1 = oi0.y - o1.y, dz1 = oi0.z - o1.z;
            const float nx0 = fmaf(dx0, iL0, 12582912.f) - 12582912.f, ny0 = fmaf(dy0, iL1, 12582912.f) - 12582912.f, nz0 = fmaf(dz0, iL2, 12582912.f) - 12582912.f;
            const float nx1 = fmaf(dx1, iL0, 12582912.f) - 12582912.f, ny1 = fmaf(dy1, iL1, 12582912.f) - 12582912.f, nz1 = fmaf(dz1, iL2, 12582912.f) - 12582912.f;
            dx0 = nb_shift(R, 0, dx0, nx0); dy0 = nb_shift(R, 1, dy0, ny0); dz0 = nb_shift(R, 2, dz0, nz0);
            dx1 = nb_shift(R, 0, dx1, nx1); dy1 = nb_shift(R, 1, dy1, ny1); dz1 = nb_shift(R, 2, dz1, nz1);
            const float r0 = dx0 * dx0 + dy0 * dy0 + dz0 * dz0, r1 = dx1 * dx1 + dy1 * dy1 + dz1 * dz1;
            const bool in0 = r0 <= rmax2, in1 = hasb && r1 <= rmax2;
            if (in0 || in1) {
                const float4 a1 = woff[3 * j0 + 1], a2 = woff[3 * j0 + 2];
                const float4 b1 = woff[3 * j1 + 1], b2 = woff[3 * j1 + 2];
                if (!in0) { dx0 = 1.0e4f; dy0 = 0.f; dz0 = 0.f; }
                if (!in1) { dx1 = 1.0e4f; dy1 = 0.f; dz1 = 0.f; }
                float2 eel = f2(0.f), elj = f2(0.f), vlj = f2(0.f);
#pragma unroll
                for (int bs = 0; bs < 3; ++bs) {
                    float2 q[3];
                    if (bs == 0) {
                        q[0] = f2(dx0, dx1); q[1] = f2(dy0, dy1); q[2] = f2(dz0, dz1);
                    } else if (bs == 1) {
                        q[0] = f2(dx0 - a1.x, dx1 - b1.x); q[1] = f2(dy0 - a1.y, dy1 - b1.y);
                        q[2] = f2(dz0 - a1.z, dz1 - b1.z);
                    } else {
                        q[0] = f2(dx0 - a2.x, dx1 - b2.x); q[1] = f2(dy0 - a2.y, dy1 - b2.y);
                        q[2] = f2(dz0 - a2.z, dz1 - b2.z);
                    }
                    float2 H[3] = {f2(0.f), f2(0.f), f2(0.f)};    // partner site bs: its gradient share
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const float2 ddx = a ? __fadd2_rn(hi[a - 1][0], q[0]) : q[0];
                        const float2 ddy = a ? __fadd2_rn(hi[a - 1][1], q[1]) : q[1];
                        const float2 ddz = a ? __fadd2_rn(hi[a - 1][2], q[2]) : q[2];
                        const float2 rr2 = __ffma2_rn(ddx, ddx, __ffma2_rn(ddy, ddy, __fmul2_rn(ddz, ddz)));
                        const float2 rinv = f2(nb_rsqrt_approx(rr2.x), nb_rsqrt_approx(rr2.y));
                        const float2 s2 = __fmul2_rn(rinv, rinv);
                        const float2 arg = __fmul2_rn(rr2, ex2c);
                        const float2 den = __ffma2_rn(palpha, __fmul2_rn(rr2, rinv), f2(1.f));
                        const float2 tt = f2(nb_rcp_approx(den.x), nb_rcp_approx(den.y));
                        const float2 u = __ffma2_rn(f2(ERFCX_A), tt, f2(ERFCX_B));
                        const float C[ERFCX_NC] = ERFCX_COEFS;
                        float2 p = f2(C[ERFCX_NC - 1]);
#pragma unroll
                        for (int m = ERFCX_NC - 2; m >= 0; --m) p = __ffma2_rn(p, u, f2(C[m]));
                        const float2 ex = f2(nb_ex2_approx(-arg.x), nb_ex2_approx(-arg.y));
                        const float2 erfcv = __fmul2_rn(ex, __fmul2_rn(tt, p));
                        const float qq = (a == 0 && bs == 0) ? qqv[0] : ((a == 0 || bs == 0) ? qqv[1] : qqv[2]);
                        const float2 e = __fmul2_rn(__fmul2_rn(f2(qq), erfcv), rinv);
                        float2 mdf = __fmul2_rn(__ffma2_rn(f2(qq * c2a), ex, e), s2);
                        if (a == 0 && bs == 0) {
                            const float2 ri = __ffma2_rn(__fmul2_rn(f2(-0.5f), rinv), __ffma2_rn(rr2, s2, f2(-1.f)), rinv);
                            const float2 sl = __fmul2_rn(ri, ri);
                            const float2 s6 = __fmul2_rn(__fmul2_rn(sl, sl), sl);
                            const float2 A = __fmul2_rn(__fmul2_rn(w12, s6), s6);
                            float2 e1 = __ffma2_rn(nw6, __ffma2_rn(s6, c6, s6), __ffma2_rn(A, c12, A));
                            float2 m1 = __fmul2_rn(__fmul2_rn(f2(6.f), sl), __ffma2_rn(nw6, s6, __fadd2_rn(A, A)));
                            if (R.lj_switch) {
                                float d0 = -m1.x, d1 = -m1.y;
                                lj_switch_apply<float>(R, rr2.x, e1.x, d0);
                                lj_switch_apply<float>(R, rr2.y, e1.y, d1);
                                m1 = f2(-d0, -d1);
                            }
                            const bool lj0 = rr2.x <= rv2, lj1 = rr2.y <= rv2;
                            e1 = f2(lj0 ? e1.x : 0.f, lj1 ? e1.y : 0.f);
                            m1 = f2(lj0 ? m1.x : 0.f, lj1 ? m1.y : 0.f);
                            elj = __fadd2_rn(elj, e1);
                            if (VIR) vlj = __fmul2_rn(m1, rr2);   // -df1 r^2 (watwat_ewald_press.f:146-152)
                            mdf = __fadd2_rn(mdf, m1);
                        }
                        eel = __fadd2_rn(eel, e);
                        G[3 * a] = __ffma2_rn(mdf, ddx, G[3 * a]);
                        G[3 * a + 1] = __ffma2_rn(mdf, ddy, G[3 * a + 1]);
                        G[3 * a + 2] = __ffma2_rn(mdf, ddz, G[3 * a + 2]);
                        H[0] = __ffma2_rn(mdf, ddx, H[0]);
                        H[1] = __ffma2_rn(mdf, ddy, H[1]);
                        H[2] = __ffma2_rn(mdf, ddz, H[2]);
                    }
                    jadd(l0, l1, j0, j1, bs, H);
                }
                const bool img0 = (nx0 != 0.f) | (ny0 != 0.f) | (nz0 != 0.f);
                const bool img1 = (nx1 != 0.f) | (ny1 != 0.f) | (nz1 != 0.f);
                e4[img0 ? 1 : 0] += elj.x;
                e4[img0 ? 3 : 2] += eel.x;
                if (VIR) e4[img0 ? NE - 1 : NE - 2] += vlj.x;
                e4[img1 ? 1 : 0] += elj.y;
                e4[img1 ? 3 : 2] += eel.y;
                if (VIR) e4[img1 ? NE - 1 : NE - 2] += vlj.y;
                npair += 18 * ((int)in0 + (int)in1);
            }
            cnt += 2;
            if (cnt >= CHUNK) { flush(2.f); cnt = 0; }
        }
        flush(2.f);
        water_vs_atoms<float>(R, i, pos, lj_v, sflags, wl2_off, wl2, cap2, g, e4, npair, flush1);
#pragma unroll
        for (int k = 0; k < 4; ++k) eu[k] = (double)sE[k][t].x + (double)sE[k][t].y;
        eu[4] = (double)npair;
        eu[6] = VIR ? (double)sE[NE - 2][t].x + (double)sE[NE - 2][t].y : 0.0;
        eu[7] = VIR ? (double)sE[NE - 1][t].x + (double)sE[NE - 1][t].y : 0.0;
    }
    __syncthreads();
    // the block's partner shares of its j-set
    const int *js = jset + (size_t)b * jcap;
    for (int l = t; l < nJ; l += HB) {
        const size_t jg = (size_t)js[l];
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            const int v = sJ[c * jcap + l];
            if (v != 0) atomicAdd((unsigned long long *)&grad[9 * jg + c], (unsigned long long)((long long)v * (1LL << (32 - S))));
        }
    }
}

// non-water atom per thread over its full site list
template <typename T>
__global__ void __launch_bounds__(128) k_atom(int nA, int nW, const RepDev *__restrict__ reps, const int *__restrict__ site_rep,
                                              const void *pos_v, const void *lj_v, const unsigned *__restrict__ sflags,
                                              const int *__restrict__ xl_off, const int *__restrict__ xl, int capx,
                                              long long *__restrict__ grad, double *__restrict__ e_unit)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nA) return;
    typedef typename vec4<T>::type T4;
    typedef typename cplx<T>::type T2;
    const T4 *pos = (const T4 *)pos_v;
    const T2 *lj = (const T2 *)lj_v;
    int si = 3 * nW + k;
    const RepDev &R = reps[site_rep[si]];
    T4 xi = pos[si];
    T2 lji = lj[si];
    unsigned fi = sflags[si];
    T g[3] = {0, 0, 0};
    long long G[3] = {0, 0, 0};
    double elp = 0, eli = 0, eep = 0, eei = 0, vp = 0, vi = 0;
    int cnt = 0, npair = 0;
    // an overflowed list is read within the buffer (the evaluation is redone)
    const int q1 = min(xl_off[k + 1], capx);
    for (int q = min(xl_off[k], capx); q < q1; ++q) {
        nb_prefetch_l1(xl + min(q + 32, q1 - 1));
        int s = xl[q];
        T4 xj = pos[s];
        T2 ljj = lj[s];
        T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        bool img;
        min_image<T>(R, dx, dy, dz, img);
        T r2 = dx * dx + dy * dy + dz * dz;
        T eel = 0, elj = 0, vir = 0;
        T df = atom_pair<T>(R, r2, xi.w, xj.w, lji.x, lji.y, ljj.x, ljj.y, fi, sflags[s], eel, elj, vir, npair);
        g[0] += df * dx; g[1] += df * dy; g[2] += df * dz;
        // LJ virial: a water partner's side of the pair (its W2 list) adds none, so it counts
        // twice here; pairs of two non-water atoms are seen from both sides
        const double wv = (double)vir * (s < 3 * nW ? 2.0 : 1.0);
        if (img) { eei += (double)eel; eli += (double)elj; vi += wv; }
        else { eep += (double)eel; elp += (double)elj; vp += wv; }
        if (++cnt == CHUNK) { flush(g, G, 3); cnt = 0; }
    }
    flush(g, G, 3);
    grad[(size_t)3 * si] = G[0];
    grad[(size_t)3 * si + 1] = G[1];
    grad[(size_t)3 * si + 2] = G[2];
    double *eu = e_unit + NB_EU * (size_t)(nW + k);
    eu[0] = elp; eu[1] = eli; eu[2] = eep; eu[3] = eei; eu[4] = (double)npair; eu[5] = 0.0;
    eu[6] = vp; eu[7] = vi;
}

// ---------------------------------------------------------------------------------
// Water exclusion corrections (cdie_ewald.f:117-199 for the O-H1, O-H2, H1-H2 pairs of each
// water), one thread per molecule, each pair once.  With u = (alpha r)^2,
//   e  = -qq erf(alpha r)/r = -qq alpha (2/sqrt(pi)) S(u),   S(u) = sum (-1)^n u^n / (n! (2n+1))
//   df = (de/dr)/r          = -qq (4 alpha^3/sqrt(pi)) S'(u)
// (Taylor series of erf, Abramowitz & Stegun 7.1.5), evaluated in FP64 with 16 terms, which
// is exact to rounding for u <= 0.5 (r <= 2.0 Å at alpha 0.35); larger u uses erf/exp.
__constant__ double c_erf_s[16] = {
    1, -0.33333333333333331, 0.10000000000000001, -0.023809523809523808, 0.0046296296296296294,
    -0.00075757575757575758, 0.00010683760683760684, -1.3227513227513228e-05, 1.4589169000933706e-06,
    -1.4503852223150468e-07, 1.3122532963802806e-08, -1.0892221037148573e-09, 8.3507027951472397e-11,
    -5.9477940136376354e-12, 3.9554295164585257e-13, -2.4668270102644571e-14};
__constant__ double c_erf_ds[15] = {
    -0.33333333333333331, 0.20000000000000001, -0.071428571428571425, 0.018518518518518517,
    -0.003787878787878788, 0.00064102564102564103, -9.2592592592592588e-05, 1.1671335200746965e-05,
    -1.3053467000835422e-06, 1.3122532963802806e-07, -1.1981443140863431e-08, 1.0020843354176688e-09,
    -7.7321322177289257e-11, 5.537601323041936e-12, -3.7002405153966856e-13};

__device__ __forceinline__ void excl_pair(double qq, double al, double rx, double ry, double rz, double &e, double &df)
{
    double r2 = rx * rx + ry * ry + rz * rz, u = al * al * r2;
    if (u <= 0.5) {
        double s = c_erf_s[15], ds = c_erf_ds[14];
#pragma unroll
        for (int k = 14; k >= 0; --k) s = fma(s, u, c_erf_s[k]);
#pragma unroll
        for (int k = 13; k >= 0; --k) ds = fma(ds, u, c_erf_ds[k]);
        e = -qq * al * NB_TWO_OVER_SQRTPI * s;
        df = -qq * 2.0 * al * al * al * NB_TWO_OVER_SQRTPI * ds;
    } else {
        double rij = sqrt(r2), sinv = 1.0 / rij, x = al * rij;
        double erfv = erf(x), derfc = NB_TWO_OVER_SQRTPI * exp(-x * x);
        e = -qq * sinv * erfv;
        df = qq * sinv * (sinv * sinv * erfv - sinv * al * derfc);
    }
}

__global__ void k_excl_water(int nW, const int *__restrict__ unit_atom, const int *__restrict__ atom_rep,
                             const RepDev *__restrict__ reps, const double *__restrict__ coor,
                             const double *__restrict__ q, double *__restrict__ grad, double *__restrict__ e_out)
{
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nW) return;
    const int a0 = unit_atom[u];
    const RepDev &R = reps[atom_rep[a0]];
    double x[3][3], qs[3], g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, ecorr = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k][0] = coor[3 * (size_t)(a0 + k)];
        x[k][1] = coor[3 * (size_t)(a0 + k) + 1];
        x[k][2] = coor[3 * (size_t)(a0 + k) + 2];
        qs[k] = q[a0 + k];
    }
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const int a = pa[p], b = pb[p];
        double rx = x[a][0] - x[b][0], ry = x[a][1] - x[b][1], rz = x[a][2] - x[b][2];
        double e, df;
        excl_pair(qs[a] * qs[b] * R.epstmp, R.alphad, rx, ry, rz, e, df);
        ecorr += e;
        g[a][0] += df * rx; g[a][1] += df * ry; g[a][2] += df * rz;
        g[b][0] -= df * rx; g[b][1] -= df * ry; g[b][2] -= df * rz;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double *gp = grad + 3 * (size_t)(a0 + k), *ep = e_out + NB_EX * (size_t)(a0 + k);
        gp[0] = g[k][0]; gp[1] = g[k][1]; gp[2] = g[k][2];
        ep[0] = k == 0 ? ecorr : 0.0; ep[1] = 0.0; ep[2] = 0.0; ep[3] = 0.0;
    }
}

// exclusion erf corrections (cdie_ewald.f:117-199) and 1-4 terms (ener14.f:38-95), FP64,
// gathered per atom over both directions; raw (unimaged) displacements as MOIL uses.
// With skip_water set, water atoms are left to k_excl_water.
__global__ void k_excl14(int natom, const int *__restrict__ atom_rep, const RepDev *__restrict__ reps,
                         const double *__restrict__ coor, const double *__restrict__ q, const int *__restrict__ ex_off,
                         const int *__restrict__ ex_j, const int *__restrict__ p_off, const int *__restrict__ p_j,
                         const double *__restrict__ p_par, const unsigned *__restrict__ aflags, int skip_water,
                         int fixed_out, double *__restrict__ grad, double *__restrict__ e_out)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natom) return;
    if (skip_water && (aflags[a] & SF_WATER)) return;
    const RepDev &R = reps[atom_rep[a]];
    double xa = coor[3 * (size_t)a], ya = coor[3 * (size_t)a + 1], za = coor[3 * (size_t)a + 2];
    double gx = 0, gy = 0, gz = 0, ecorr = 0, eel14 = 0, evdw14 = 0, vir14 = 0;
    double qa = q[a] * R.epstmp, al = R.alphad;
    for (int k = ex_off[a]; k < ex_off[a + 1]; ++k) {
        int b = ex_j[k];
        double rx = xa - coor[3 * (size_t)b], ry = ya - coor[3 * (size_t)b + 1], rz = za - coor[3 * (size_t)b + 2];
        double r2 = rx * rx + ry * ry + rz * rz, s2 = 1.0 / r2, rij = sqrt(r2), s = 1.0 / rij;
        double qq = qa * q[b], x = al * rij;
        double erfv = erf(x), derfc = NB_TWO_OVER_SQRTPI * exp(-x * x);
        double e2 = -qq * s * erfv;
        double df = qq * s * (s2 * erfv - s * al * derfc);
        gx += df * rx; gy += df * ry; gz += df * rz;
        ecorr += 0.5 * e2;
    }
    for (int k = p_off[a]; k < p_off[a + 1]; ++k) {
        int b = p_j[k];
        const double *p = p_par + 3 * (size_t)k;
        double rx = xa - coor[3 * (size_t)b], ry = ya - coor[3 * (size_t)b + 1], rz = za - coor[3 * (size_t)b + 2];
        double r2 = rx * rx + ry * ry + rz * rz, s2 = 1.0 / r2, e1 = 0, df1 = 0, e2 = 0, df2 = 0;
        if (p[0] > 1e-12) {
            double s6 = s2 * s2 * s2, A = p[0] * s6 * s6, B = p[1] * s6;
            e1 = A - B;
            df1 = -6.0 * s2 * (A + e1);
            vir14 -= 0.5 * df1 * r2;   // ener14_press.f:51-59
        }
        if (fabs(p[2]) > 1e-12) {
            double s = sqrt(s2);
            e2 = p[2] * s;
            df2 = -e2 * s2;
        }
        double df = df1 + df2;
        gx += df * rx; gy += df * ry; gz += df * rz;
        evdw14 += 0.5 * e1;
        eel14 += 0.5 * e2;
    }
    if (fixed_out) {   // mixed path: 2^32 fixed point, as the site gradients
        long long *gf = (long long *)grad + 3 * (size_t)a;
        gf[0] = __double2ll_rn(gx * NB_FIX_SCALE);
        gf[1] = __double2ll_rn(gy * NB_FIX_SCALE);
        gf[2] = __double2ll_rn(gz * NB_FIX_SCALE);
    } else {
        grad[3 * (size_t)a] = gx; grad[3 * (size_t)a + 1] = gy; grad[3 * (size_t)a + 2] = gz;
    }
    double *eo = e_out + NB_EX * (size_t)a;
    eo[0] = ecorr; eo[1] = eel14; eo[2] = evdw14; eo[3] = vir14;
}

// ---------------------------------------------------------------------------------
// gradient assembly in MOIL order: fixed-point real space + FP64 corrections + PME
template <typename T>
__global__ void k_final_grad(int natom, const int *__restrict__ site_of, const int *__restrict__ atom_rep,
                             const RepDev *__restrict__ reps, const long long *__restrict__ grad_site,
                             const double *__restrict__ grad_ex, const T *__restrict__ part,
                             const double *__restrict__ q, int nsw, double *__restrict__ dpot, int *st)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natom) return;
    const RepDev &R = reps[atom_rep[a]];
    int s = site_of[a];
    bool bad = false;
    if constexpr (sizeof(T) == 4) {
        // FP32 path: the PME share (one float4 per site from k_pme_gather_f) is scaled in
        // FP32 (its own precision) and joins the fixed-point real-space and correction terms
        // as an integer; the double result is assembled with integer operations (no FP64
        // instruction).  Sites below nsw (waters whose corrections the water kernel added)
        // have no correction term.
        const long long *gx = (const long long *)grad_ex + 3 * (size_t)a;
        const bool ex = s >= nsw;
        const float qs = (float)q[a];
        const float4 p4 = ((const float4 *)part)[s];
        const float pg[3] = {p4.x, p4.y, p4.z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const long long v = grad_site[3 * (size_t)s + d] + (ex ? gx[d] : 0LL) + nb_f2fix(qs * R.pme_gs[d] * pg[d]);
            bad |= (v > (1LL << 61)) | (v < -(1LL << 61));   // a saturated (non-finite) term
            dpot[3 * (size_t)a + d] = nb_fix2d(v);
        }
    } else {
        const T *p = part + 12 * (size_t)s;   // 4 plane slots per site (k_plane_inv)
        double pg[3] = {0, 0, 0};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            pg[0] += (double)p[3 * t];
            pg[1] += (double)p[3 * t + 1];
            pg[2] += (double)p[3 * t + 2];
        }
        double qf = q[a] * R.fcd;
        double sc[3] = {qf * R.n1 * R.invLd[0], qf * R.n2 * R.invLd[1], qf * R.n3 * R.invLd[2]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double v = (double)grad_site[3 * (size_t)s + d] * NB_FIX_INV + grad_ex[3 * (size_t)a + d] + sc[d] * pg[d];
            bad |= !(v == v);
            dpot[3 * (size_t)a + d] = v;
        }
    }
    if (bad) atomicOr(&st[1], NB_DEV_ERR_NAN);
}

// Per-replica energies in two passes with a fixed partition, so large replicas spread over
// many blocks and the sums stay in a fixed order (deterministic):
//  k_energy_part: one block per chunk (EChunk: up to NB_FE_SEG consecutive units, atoms or PME
//    column items of one replica); every thread streams the chunk's flat array with a stride
//    that keeps its slot fixed (coalesced reads), the slots are summed by a halving tree;
//  k_energy_final: one thread per replica adds its chunks' slot sums in chunk order and forms
//    MOIL's energy names (pot/eforce.f:122-204).
#define NB_FE_THREADS 256
static_assert(NB_FE_THREADS % NB_EU == 0 && NB_FE_THREADS % NB_EX == 0, "slot-preserving stride");
__global__ void __launch_bounds__(NB_FE_THREADS) k_energy_part(const EChunk *__restrict__ chunks,
                                                               const double *__restrict__ e_unit,
                                                               const double *__restrict__ e_ex,
                                                               const double *__restrict__ e_col,
                                                               double *__restrict__ part)
{
    __shared__ double sh[NB_FE_THREADS];
    const int t = threadIdx.x;
    const EChunk ch = chunks[blockIdx.x];
    const int width = ch.kind <= 1 ? NB_EU : (ch.kind == 2 ? NB_EX : 1);
    const double *b = ch.kind <= 1 ? e_unit + (size_t)NB_EU * ch.begin
                                   : (ch.kind == 2 ? e_ex + (size_t)NB_EX * ch.begin : e_col + ch.begin);
    const int n = width * (ch.end - ch.begin);
    // four loads in flight per thread, four partial sums added in a fixed order
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    int k = t;
    for (; k + 3 * NB_FE_THREADS < n; k += 4 * NB_FE_THREADS) {
#pragma unroll
        for (int j = 0; j < 4; ++j) p[j] += b[k + j * NB_FE_THREADS];
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
        if (k + j * NB_FE_THREADS < n) p[j] += b[k + j * NB_FE_THREADS];
    sh[t] = (p[0] + p[1]) + (p[2] + p[3]);
    __syncthreads();
    // halving tree while the live range halves into a multiple of the slot width (thread k
    // adds k + half, which holds the same slot)
    int live = NB_FE_THREADS;
    while (live % 2 == 0 && (live / 2) % width == 0) {
        const int h = live / 2;
        if (t < h) sh[t] += sh[t + h];
        __syncthreads();
        live = h;
    }
    if (t < NB_EU) {
        double w = 0.0;
        if (t < width)
            for (int q = t; q < live; q += width) w += sh[q];
        part[(size_t)NB_EU * blockIdx.x + t] = w;
    }
}

__global__ void k_energy_final(int nrep, const RepDev *__restrict__ reps, const EChunk *__restrict__ chunks,
                               const int *__restrict__ chunk_begin, const double *__restrict__ part,
                               double *__restrict__ e_rep)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrep) return;
    const RepDev &R = reps[r];
    double pw[NB_EU] = {0, 0, 0, 0, 0, 0, 0, 0}, po[NB_EU] = {0, 0, 0, 0, 0, 0, 0, 0};
    double px[NB_EX] = {0, 0, 0, 0}, cl = 0.0;
    for (int c = chunk_begin[r]; c < chunk_begin[r + 1]; ++c) {
        const double *q = part + (size_t)NB_EU * c;
        const int kind = chunks[c].kind;
        if (kind == 0) { for (int k = 0; k < NB_EU; ++k) pw[k] += q[k]; }
        else if (kind == 1) { for (int k = 0; k < NB_EU; ++k) po[k] += q[k]; }
        else if (kind == 2) { for (int k = 0; k < NB_EX; ++k) px[k] += q[k]; }
        else cl += q[0];
    }
    const double elp = 0.5 * (pw[0] + po[0]), eli = 0.5 * (pw[1] + po[1]);
    const double eep = 0.5 * (pw[2] + po[2]), eei = 0.5 * (pw[3] + po[3]);
    const double npairs = 0.5 * (pw[4] + po[4]);
    // waters relative to the reference water (k_wref) add their reference energy here
    const double ecorr = px[0] + pw[5] + po[5] + (R.wref ? (double)R.nwat * R.wcorr0 : 0.0);
    const double eel14 = px[1], evdw14 = px[2];
    const double erec = 0.5 * cl;
    double *o = e_rep + NB_EREP * (size_t)r;
    o[0] = elp; o[1] = eep; o[2] = eli; o[3] = eei;          // e_vdw, e_el, e_vsym, e_lsym
    o[4] = eel14; o[5] = evdw14; o[6] = ecorr; o[7] = R.e_self; o[8] = erec;
    o[9] = elp + eep + eli + eei + eel14 + evdw14 + ecorr + R.e_self + erec;
    o[10] = eep + eei;
    o[11] = npairs;                                           // in-cutoff site pairs
    // LJ virial terms virvdw1..5 (MOIL's PRESS build): water-water primary and images,
    // other pairs primary and images, 1-4
    o[12] = 0.5 * pw[6]; o[13] = 0.5 * pw[7]; o[14] = 0.5 * po[6]; o[15] = 0.5 * po[7]; o[16] = px[3];
}

// the half-list kernel for a block size (128, 256 or 512 waters) and virial flag
using WaterHFn = decltype(&k_water_h<256, false>);
WaterHFn water_h_fn(int hb, bool vir)
{
    switch (hb) {
    case 128: return vir ? k_water_h<128, true> : k_water_h<128, false>;
    case 512: return vir ? k_water_h<512, true> : k_water_h<512, false>;
    default: return vir ? k_water_h<256, true> : k_water_h<256, false>;
    }
}

template <typename T>
void realspace_t(NbCtx *c)
{
    cudaStream_t s = c->stream;
    if (c->timing) cudaEventRecord(c->ev[2], s);
    if (sizeof(T) == 4 && c->nW > 0 && c->whalf) {
        // the water sites' gradients are sums of atomics: cleared first
        cudaMemsetAsync(c->d_grad_site, 0, sizeof(long long) * 9 * (size_t)c->nW, s);
        water_h_fn(c->hb, c->virial)<<<(int)c->hblocks.size(), c->hb, (size_t)36 * c->jcap, s>>>(
            c->d_hblocks, c->d_reps, (const float4 *)c->d_pos, (const float4 *)c->d_woff, c->d_site_lj,
            c->d_site_flags, c->d_hrow, c->caph, c->d_hcnt, c->d_jset, c->d_jn, c->jcap, c->d_wl2_off, c->d_wl2,
            cap_int(c->cap_wl2), c->d_grad_site, c->d_e_unit, c->water_excl_fast);
        c->launches++;
    } else if (c->nW > 0) {
        const int nb = (int)((c->nW + WBLOCK - 1) / WBLOCK);
        if constexpr (sizeof(T) == 4)
            (c->virial ? (c->row16 ? k_water_f<true, unsigned short> : k_water_f<true, int>)
                       : (c->row16 ? k_water_f<false, unsigned short> : k_water_f<false, int>))<<<nb, WBLOCK, 0, s>>>(
                (int)c->nW, c->d_reps, c->d_site_rep, (const float4 *)c->d_pos, (const float4 *)c->d_woff,
                c->d_site_lj, c->d_site_flags, c->d_wl1_cnt, c->d_wl1, c->cap_row1, c->d_wl2_off, c->d_wl2,
                cap_int(c->cap_wl2), c->d_grad_site, c->d_e_unit, c->water_excl_fast);
        else
            (c->row16 ? k_water<T, unsigned short> : k_water<T, int>)<<<(int)((c->nW + WBLOCK64 - 1) / WBLOCK64), WBLOCK64, 0, s>>>((int)c->nW, c->d_reps, c->d_site_rep, c->d_pos, c->d_woff,
                                             c->d_site_lj, c->d_site_flags, c->d_wl1_cnt, c->d_wl1, c->cap_row1,
                                             c->d_wl2_off, c->d_wl2, cap_int(c->cap_wl2), c->d_grad_site,
                                             c->d_e_unit);
        c->launches++;
    }
    if (c->timing) cudaEventRecord(c->ev[3], s);
    if (c->nA > 0) {
        k_atom<T><<<(int)((c->nA + 127) / 128), 128, 0, s>>>((int)c->nA, (int)c->nW, c->d_reps, c->d_site_rep,
                                                             c->d_pos, c->d_site_lj, c->d_site_flags, c->d_xl_off,
                                                             c->d_xl, cap_int(c->cap_xl), c->d_grad_site, c->d_e_unit);
        c->launches++;
    }
    if (c->timing) cudaEventRecord(c->ev[4], s);
}

}  // namespace

void nb_launch_realspace(NbCtx *c)
{
    if (c->precision == MOIL_NB_FP64) realspace_t<double>(c);
    else realspace_t<float>(c);
}

// shared-memory carveout (percent of the per-SM maximum) for `bytes` of resident blocks
static int carveout_pct(NbCtx *c, size_t bytes)
{
    int smax = 0;
    if (cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device) != cudaSuccess || smax <= 0)
        return 100;
    return (int)std::min<size_t>(100, (100 * bytes + smax - 1) / smax);
}

int nb_realspace_configure(NbCtx *c)
{
    // full-list FP32 water kernels: four resident blocks of static shared memory each; the
    // smallest carveout that holds them leaves the most L1 for the partner-record gathers
    const void *fns[4] = {(const void *)k_water_f<false, unsigned short>, (const void *)k_water_f<false, int>,
                          (const void *)k_water_f<true, unsigned short>, (const void *)k_water_f<true, int>};
    for (const void *fn : fns) {
        cudaFuncAttributes fa;
        NB_CUDA_OK(c, cudaFuncGetAttributes(&fa, fn));
        NB_CUDA_OK(c, cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                           carveout_pct(c, 4 * fa.sharedSizeBytes)));
    }
    return MOIL_NB_OK;
}

// the half-list kernel keeps two resident blocks per SM (its register budget) with the
// current j-set capacity
bool nb_half_two_blocks(NbCtx *c)
{
    int smax = 0;
    cudaFuncAttributes fa;
    const void *fn = (const void *)water_h_fn(c->hb, false);
    if (cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, fn) != cudaSuccess)
        return false;
    const int per_sm = 512 / c->hb;
    return (size_t)per_sm * ((size_t)36 * c->jcap + fa.sharedSizeBytes + 1024) <= (size_t)smax;
}

int nb_half_configure(NbCtx *c)
{
    int optin = 0;
    NB_CUDA_OK(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const void *fns[2] = {(const void *)water_h_fn(c->hb, false), (const void *)water_h_fn(c->hb, true)};
    const size_t dyn = (size_t)36 * c->jcap;
    for (const void *fn : fns) {
        cudaFuncAttributes fa;
        NB_CUDA_OK(c, cudaFuncGetAttributes(&fa, fn));
        if (c->jcap > 65535 || dyn + fa.sharedSizeBytes > (size_t)optin) return MOIL_NB_ERR_OVERFLOW;
        // the limit belongs to the kernel, not to the handle: other handles (replica groups)
        // may launch it with larger j-sets, so it only ever grows
        if ((int)dyn > fa.maxDynamicSharedSizeBytes)
            NB_CUDA_OK(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        // the smallest shared-memory carveout that holds the resident blocks (512 / hb per SM):
        // the rest of the SM's unified memory stays L1 for the partner-record gathers
        NB_CUDA_OK(c, cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                           carveout_pct(c, (512 / c->hb) * (dyn + fa.sharedSizeBytes))));
    }
    return MOIL_NB_OK;
}

void nb_launch_excl14(NbCtx *c, const double *d_coor)
{
    const int fast = c->water_excl_fast && c->nW > 0;
    // mixed path: the water kernel adds each water's own corrections (k_water_f)
    if (fast && c->precision == MOIL_NB_FP64) {
        k_excl_water<<<(int)((c->nW + 127) / 128), 128, 0, c->stream>>>(
            (int)c->nW, c->d_unit_atom, c->d_atom_rep, c->d_reps, d_coor, c->d_q, c->d_grad_ex, c->d_e_ex);
        c->launches++;
    }
    if (!fast || c->nA > 0) {
        k_excl14<<<(int)((c->natom + 127) / 128), 128, 0, c->stream>>>(
            (int)c->natom, c->d_atom_rep, c->d_reps, d_coor, c->d_q, c->d_ex_off, c->d_ex_j, c->d_p14_off,
            c->d_p14_j, c->d_p14_par, c->d_aflags, fast, c->precision != MOIL_NB_FP64, c->d_grad_ex, c->d_e_ex);
        c->launches++;
    }
}

void nb_launch_finalize(NbCtx *c, double *d_dpot)
{
    cudaStream_t s = c->stream;
    if (c->precision == MOIL_NB_FP64)
        k_final_grad<double><<<(int)((c->natom + 255) / 256), 256, 0, s>>>(
            (int)c->natom, c->d_site_of, c->d_atom_rep, c->d_reps, c->d_grad_site, c->d_grad_ex,
            (const double *)c->d_part, c->d_q, 0, d_dpot, c->d_status);
    else
        k_final_grad<float><<<(int)((c->natom + 255) / 256), 256, 0, s>>>(
            (int)c->natom, c->d_site_of, c->d_atom_rep, c->d_reps, c->d_grad_site, c->d_grad_ex,
            (const float *)c->d_part, c->d_q, c->water_excl_fast ? (int)(3 * c->nW) : 0, d_dpot, c->d_status);
    k_energy_part<<<(int)c->echunks.size(), NB_FE_THREADS, 0, s>>>(c->d_echunks, c->d_e_unit, c->d_e_ex, c->d_e_col,
                                                                    c->d_epart);
    k_energy_final<<<(c->nrep + 127) / 128, 128, 0, s>>>(c->nrep, c->d_reps, c->d_echunks, c->d_echunk_begin,
                                                         c->d_epart, c->d_e_rep);
    c->launches += 3;
}
