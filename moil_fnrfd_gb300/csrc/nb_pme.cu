// nb_pme.cu -- PME reciprocal sum (pot/ewald_receip.f:101-1080), GB300 layout.
//
// The reference spreads into a padded complex grid, runs two full 3D C2C FFTs
// (pubz3d / FFTPACK) with the influence function in between (scalar_sum) and gathers.
// Here the real-space charge grid never exists in HBM:
//   k_pme_bin      fractional coordinates fr = n (w - anint(w) + 1/2) (:250-260), atoms
//                  bucketed by int(fr3) (the last z plane of their stencil)
//   plane_fwd      one CTA per (replica, z plane): the 4x4 x-y stencils of every atom whose
//                  z stencil touches the plane are accumulated in shared memory in 64-bit
//                  fixed point (order independent, hence deterministic), then R2C along x
//                  and C2C along y in shared memory; the half-complex plane goes to HBM
//                  as [z][kx][ky]
//   zconv          one CTA per (replica, kx, run of ky): C2C along z, the influence function
//                  exp(-pi^2 m^2 / alpha^2) / (pi V B(m) m^2) with the FP64 energy sum
//                  (scalar_sum, :723-812), inverse C2C along z, written back in place
//   plane_inv      one CTA per (replica, z plane): inverse C2C along y, C2R along x in shared
//                  memory, then each atom's share of the gradient from this plane (grad_sum,
//                  :815-970) into its own slot -- four planes, four slots, summed at the end
// FFTs (FP32 path): Stockham autosort with radices 2..5 (plane kernels) or up to 10 (z
// columns, two passes per line: the composite codelets of nb_fft.cuh); every pass transforms all lines
// of a tile at once, the block's threads spread over (line, butterfly) pairs, with the
// index arithmetic (twiddle step, destination) read from per-stage tables built on the host
// and the line number obtained by a multiply-high by a precomputed magic constant.  The
// last pass of a direction stores transposed, so the next direction reads contiguous lines.
// The plain FP64 path uses a simpler one-warp-per-line FFT with the same layout.
// Inverse transforms are conj(FFT(conj(x))), unnormalised like FFTPACK's cfftb.
#include <mutex>

#include "nb_fft.cuh"
#include "nb_internal.h"

namespace {

__device__ __forceinline__ float nb_round(float x) { return roundf(x); }
__device__ __forceinline__ double nb_round(double x) { return round(x); }

__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// ---------------------------------------------------------------------------------
// binning (both precisions)

template <typename T>
__global__ void k_pme_bin(int nsite, const int *__restrict__ site_rep, const RepDev *__restrict__ reps,
                          const void *pos_v, const void *q_v, void *fr_v, int *__restrict__ zcount,
                          int *__restrict__ zslot)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    typedef typename vec4<T>::type T4;
    const RepDev &R = reps[site_rep[s]];
    T4 p = ((const T4 *)pos_v)[s];
    T4 o;
    int zb;
    if constexpr (sizeof(T) == 4) {
        // fr = n (u - anint(u) + 1/2), u = x / L, carried as hi + lo through every step (1/L as
        // hi + lo, the product's rounding error by an FMA, the + 1/2 by Fast2Sum) so the
        // fraction within the grid cell keeps 2^-23 of a grid spacing
        const float xs[3] = {p.x, p.y, p.z};
        const int ns[3] = {R.n1, R.n2, R.n3};
        float out[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float x = xs[d], ih = R.invL[d];
            const float uh = x * ih, ul = fmaf(x, ih, -uh) + x * R.invL_lo[d];
            const float a = uh - rintf(uh);              // exact (Sterbenz)
            const float th = a + 0.5f, tl = (a - (th - 0.5f)) + ul;
            const float n = (float)ns[d];
            int i = (int)floorf(n * th);
            float w = fmaf(n, th, -(float)i) + n * tl;
            if (w < 0.f) { --i; w += 1.f; }
            if (w >= 1.f) { ++i; w -= 1.f; }
            if (i < 0) { i = 0; w = 0.f; }
            out[d] = pme_fr_pack(i, w);
            if (d == 2) zb = i;
        }
        o.x = out[0]; o.y = out[1]; o.z = out[2];
        o.w = ((const T *)q_v)[s] * (T)R.fc;
    } else {
        T w, f1, f2, f3;
        w = p.x * rep_invL<T>(R, 0); f1 = (T)R.n1 * (w - nb_round(w) + (T)0.5);
        w = p.y * rep_invL<T>(R, 1); f2 = (T)R.n2 * (w - nb_round(w) + (T)0.5);
        w = p.z * rep_invL<T>(R, 2); f3 = (T)R.n3 * (w - nb_round(w) + (T)0.5);
        o.x = f1; o.y = f2; o.z = f3;
        o.w = ((const T *)q_v)[s] * (T)R.fcd;
        zb = (int)f3;
    }
    ((T4 *)fr_v)[s] = o;
    zb = zb >= R.n3 ? zb - R.n3 : (zb < 0 ? 0 : zb);
    // one atomic per distinct bin of the warp (a warp's sites are neighbours in space)
    const int key = R.zb0 + zb, lane = threadIdx.x & 31;
    const unsigned same = __match_any_sync(__activemask(), key);
    const int leader = __ffs(same) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&zcount[key], __popc(same));
    base = __shfl_sync(same, base, leader);
    zslot[s] = base + __popc(same & ((1u << lane) - 1));
}

__global__ void k_pme_scatter(int nsite, const int *__restrict__ site_rep, const RepDev *__restrict__ reps,
                              const void *fr_v, int is_double, const int *__restrict__ zstart,
                              const int *__restrict__ zslot, int *__restrict__ zatoms)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    const RepDev &R = reps[site_rep[s]];
    int zb;
    if (is_double) zb = (int)((const double4 *)fr_v)[s].z;
    else zb = __float_as_int(((const float4 *)fr_v)[s].z) >> 23;   // pme_fr_split
    zb = zb >= R.n3 ? zb - R.n3 : (zb < 0 ? 0 : zb);
    zatoms[zstart[R.zb0 + zb] + zslot[s]] = s;
}

// plane accumulation.  FP32: int32 fixed point; the caller pre-multiplies by the replica's
// spread_scale (nb_spread_exp) so one contribution stays below 2^25 and rounds it to the
// nearest integer.  Integer addition makes the plane independent of the order of the
// atomics.  FP64: FP64 atomics.
template <typename T> struct Acc;
template <> struct Acc<float> {
    typedef int type;
    __device__ static void add(type *p, float x) { atomicAdd(p, __float2int_rn(x)); }
    __device__ static float get(type v, float inv) { return __int2float_rn(v) * inv; }
};
template <> struct Acc<double> {
    typedef double type;
    __device__ static void add(type *p, double v) { atomicAdd(p, v); }
    __device__ static double get(type v, double) { return v; }
};

// Order-4 weights of fractional offset w in closed form (the cardinal cubic B-spline that
// fill_bspline's recursion evaluates, ewald_receip.f:1022-1080):
//   th = ((1-w)^3, 4 - 6w^2 + 3w^3, 1 + 3w + 3w^2 - 3w^3, w^3) / 6
//   dth = (-(1-w)^2, 3w^2 - 4w, 1 + 2w - 3w^2, w^2) / 2
template <typename T>
__device__ __forceinline__ void bsp4_th(T w, T th[4])
{
    const T w2 = w * w, w3 = w2 * w, m = (T)1 - w, s = (T)(1.0 / 6.0);
    th[0] = s * m * m * m;
    th[1] = s * ((T)4 - (T)6 * w2 + (T)3 * w3);
    th[2] = s * ((T)1 + (T)3 * (w + w2 - w3));
    th[3] = s * w3;
}
// 6 th: the same weights without the factor 1/6, whose FP32 rounding (2.98e-8 high) would
// raise every spread charge by 9e-8 and the reciprocal energy by 1.8e-7; the FP32 spread
// applies 1/216 once per site (spread216)
__device__ __forceinline__ void bsp4_th6(float w, float th[4])
{
    const float w2 = w * w, w3 = w2 * w, m = 1.f - w;
    th[0] = m * m * m;
    th[1] = 4.f - 6.f * w2 + 3.f * w3;
    th[2] = 1.f + 3.f * (w + w2 - w3);
    th[3] = w3;
}
template <typename T>
__device__ __forceinline__ void bsp4_dth(T w, T d[4])
{
    const T w2 = w * w, m = (T)1 - w;
    d[0] = (T)-0.5 * m * m;
    d[1] = (T)0.5 * w * ((T)3 * w - (T)4);
    d[2] = (T)0.5 * ((T)1 + (T)2 * w - (T)3 * w2);
    d[3] = (T)0.5 * w2;
}
// grid index i in [-3, n] wrapped into [0, n)
__device__ __forceinline__ int pme_wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// the 4x4 x-y stencil of every atom whose z stencil reaches plane z; one atom per thread
template <typename T>
__device__ __forceinline__ void spread_plane(const RepDev &R, int z, const int *__restrict__ zstart,
                                             const int *__restrict__ zatoms, const typename vec4<T>::type *fr,
                                             typename Acc<T>::type *acc, T scale)
{
    typedef typename vec4<T>::type T4;
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3;
    for (int tp = 0; tp < 4; ++tp) {
        int zb = z + tp;
        zb = zb >= n3 ? zb - n3 : zb;
        const int b0 = zstart[R.zb0 + zb], b1 = zstart[R.zb0 + zb + 1];
        const int t3 = 3 - tp;
        for (int idx = b0 + threadIdx.x; idx < b1; idx += blockDim.x) {
            const T4 f = fr[zatoms[idx]];
            int i1, i2, i3;
            T w1, w2, w3;
            pme_fr_split(f.x, i1, w1);
            pme_fr_split(f.y, i2, w2);
            pme_fr_split(f.z, i3, w3);
            T th1[4], th2[4], th3[4];
            if constexpr (sizeof(T) == 4) {
                bsp4_th6(w1, th1);
                bsp4_th6(w2, th2);
                bsp4_th6(w3, th3);
            } else {
                bsp4_th<T>(w1, th1);
                bsp4_th<T>(w2, th2);
                bsp4_th<T>(w3, th3);
            }
            const T qz = th3[t3] * (f.w * scale);
            int xs[4];
#pragma unroll
            for (int t1 = 0; t1 < 4; ++t1) xs[t1] = pme_wrap(i1 - 3 + t1, n1);
#pragma unroll
            for (int t2 = 0; t2 < 4; ++t2) {
                typename Acc<T>::type *row = acc + pme_wrap(i2 - 3 + t2, n2) * n1;
                const T v = th2[t2] * qz;
#pragma unroll
                for (int t1 = 0; t1 < 4; ++t1) Acc<T>::add(row + xs[t1], v * th1[t1]);
            }
        }
    }
}

// gradient share of plane z (real values Rp[ky][x]) for the atoms whose z stencil reaches it
template <typename T>
__device__ __forceinline__ void gather_plane(const RepDev &R, int z, const int *__restrict__ zstart,
                                             const int *__restrict__ zatoms, const typename vec4<T>::type *fr,
                                             const T *Rp, T *__restrict__ part, bool pot = false)
{
    typedef typename vec4<T>::type T4;
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3;
    for (int tp = 0; tp < 4; ++tp) {
        int zb = z + tp;
        zb = zb >= n3 ? zb - n3 : zb;
        const int b0 = zstart[R.zb0 + zb], b1 = zstart[R.zb0 + zb + 1];
        const int t3 = 3 - tp;
        for (int idx = b0 + threadIdx.x; idx < b1; idx += blockDim.x) {
            const int s = zatoms[idx];
            const T4 f = fr[s];
            int i1, i2, i3;
            T w1, w2, w3;
            pme_fr_split(f.x, i1, w1);
            pme_fr_split(f.y, i2, w2);
            pme_fr_split(f.z, i3, w3);
            T th1[4], dt1[4], th2[4], dt2[4], th3[4], dt3[4];
            bsp4_th<T>(w1, th1); bsp4_dth<T>(w1, dt1);
            bsp4_th<T>(w2, th2); bsp4_dth<T>(w2, dt2);
            bsp4_th<T>(w3, th3); bsp4_dth<T>(w3, dt3);
            int xs[4];
#pragma unroll
            for (int t1 = 0; t1 < 4; ++t1) xs[t1] = pme_wrap(i1 - 3 + t1, n1);
            T gx = 0, gy = 0, gz = 0;
#pragma unroll
            for (int t2 = 0; t2 < 4; ++t2) {
                const T *row = Rp + pme_wrap(i2 - 3 + t2, n2) * n1;
                T sx = 0, sy = 0;
#pragma unroll
                for (int t1 = 0; t1 < 4; ++t1) {
                    const T q = row[xs[t1]];
                    sx += q * dt1[t1];
                    sy += q * th1[t1];
                }
                gx += sx * th2[t2];
                gy += sy * dt2[t2];
                gz += sy * th2[t2];
            }
            if (pot) {
                // the potential share of this plane (parameter derivatives): one slot per plane
                part[4 * (size_t)s + t3] = gz * th3[t3];
                continue;
            }
            T *o = part + 12 * (size_t)s + 3 * t3;
            o[0] = gx * th3[t3];
            o[1] = gy * th3[t3];
            o[2] = gz * dt3[t3];
        }
    }
}

// influence function (scalar_sum): m folded as MOIL does (k > ceil(n/2) - 1 -> k - n)
template <typename T>
__device__ __forceinline__ T eterm_of(const RepDev &R, const T *bsp, int kx, int ky, int kz)
{
    if (kx == 0 && ky == 0 && kz == 0) return (T)0;
    const int nf2 = (R.n2 + 1) / 2, nf3 = (R.n3 + 1) / 2;
    int m2 = ky < nf2 ? ky : ky - R.n2, m3 = kz < nf3 ? kz : kz - R.n3;
    T mh1 = (T)kx * rep_invL<T>(R, 0), mh2 = (T)m2 * rep_invL<T>(R, 1), mh3 = (T)m3 * rep_invL<T>(R, 2);
    T msq = mh1 * mh1 + mh2 * mh2 + mh3 * mh3;
    return exp(-(T)R.pme_fac * msq) /
           ((T)R.pivol * bsp[kx] * bsp[R.n1 + ky] * bsp[R.n1 + R.n2 + kz] * msq);
}

// =================================================================================
// FP32 path: block-cooperative table-driven Stockham passes

#define NB_TKF 32     // z lines per zconv CTA (FP32 path)

// Shared-memory layout of the intermediate results between Stockham stages: element e of a
// buffer is stored at e + e/16 (one spare slot per 16 float2, i.e. per 128 bytes), so the
// strided stores of the early stages (stride R for radix R) and the strided reads of the
// later ones spread over all banks.  Inputs and outputs of a transform keep the caller's
// layout.
__host__ __device__ __forceinline__ int swz(int e) { return e + (e >> 4); }
// float2 slots that hold m elements in the spread layout
__host__ __device__ __forceinline__ int swz_elems(int m) { return m + (m >> 4) + 1; }

// One Stockham stage over L lines of length n.  Source line l at src + l*ss (contiguous),
// or in the spread layout (SW_IN).  Destination: MODE 0 natural (dst + l*ds, spread if
// SW_OUT), MODE 1 transposed (dst[k*ds + l] for k < keep), MODE 2 real part natural
// (rdst + l*ds).  CONJ_OUT conjugates the stored values.  tab / tw point into shared memory
// (fft_ctx_load).
template <int RADIX, int MODE, bool CONJ_OUT, bool SW_IN, bool SW_OUT>
__device__ __forceinline__ void fft_pass_r(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                           float *__restrict__ rdst, int L, int ss, int ds, int keep,
                                           int Ns, int nb, unsigned magic, const int2 *__restrict__ tab,
                                           const float2 *__restrict__ tw)
{
    const int total = L * nb;
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        int line = nb == 1 ? b : (int)__umulhi((unsigned)b, magic);
        int j = b - line * nb;
        int2 e = tab[j];
        const int s0 = line * ss + j;
        float2 v[RADIX];
#pragma unroll
        for (int r = 0; r < RADIX; ++r) v[r] = src[SW_IN ? swz(s0 + r * nb) : s0 + r * nb];
#pragma unroll
        for (int r = 1; r < RADIX; ++r) v[r] = cmul(v[r], tw[r * e.x]);
        bfly<RADIX>(v);
#pragma unroll
        for (int r = 0; r < RADIX; ++r) {
            float2 o = CONJ_OUT ? cconj(v[r]) : v[r];
            int k = e.y + r * Ns;
            if (MODE == 0) { const int d = line * ds + k; dst[SW_OUT ? swz(d) : d] = o; }
            else if (MODE == 1) { if (k < keep) dst[k * ds + line] = o; }
            else rdst[line * ds + k] = o.x;
        }
    }
    __syncthreads();
}

// WIDE: the radix set of a wide plan (2..10); otherwise 2, 3, 4, 5 only, so the kernel keeps
// the register count of the small butterflies
template <int MODE, bool CONJ_OUT, bool SW_IN, bool SW_OUT, bool WIDE>
__device__ __forceinline__ void fft_pass(int R, const float2 *src, float2 *dst, float *rdst, int L, int ss, int ds,
                                         int keep, int Ns, int nb, unsigned magic, const int2 *tab, const float2 *tw)
{
    switch (R) {
    case 4: fft_pass_r<4, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
    case 2: fft_pass_r<2, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
    case 3: fft_pass_r<3, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
    case 5: fft_pass_r<5, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
    default:
        if constexpr (WIDE) {
            switch (R) {
            case 6: fft_pass_r<6, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
            case 8: fft_pass_r<8, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
            case 9: fft_pass_r<9, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
            default: fft_pass_r<10, MODE, CONJ_OUT, SW_IN, SW_OUT>(src, dst, rdst, L, ss, ds, keep, Ns, nb, magic, tab, tw); break;
            }
        }
        break;
    }
}

// A plan with its stage table and twiddles, staged in shared memory by fft_ctx_load so the
// butterflies read them without global-memory latency.
struct FftCtx {
    const FftPlanDev *p;
    const int2 *tab;      // plan-local: stage s at tab + p->off[s]
    const float2 *tw;     // plan-local twiddles, n entries
};

// shared-memory bytes of one staged plan of length n
size_t fft_ctx_bytes(int n, bool wide);

__device__ __forceinline__ unsigned char *fft_ctx_load(unsigned char *dst, const FftPlanDev *__restrict__ gp,
                                                       const int2 *__restrict__ gtab, const float2 *__restrict__ gtw,
                                                       FftCtx &ctx)
{
    const int n = gp->n, nst = gp->nst;
    const int ntab = gp->off[nst - 1] + gp->nb[nst - 1];
    FftPlanDev *sp = (FftPlanDev *)dst;
    int2 *st = (int2 *)(dst + align16(sizeof(FftPlanDev)));
    float2 *stw = (float2 *)((unsigned char *)st + align16(ntab * sizeof(int2)));
    for (int k = threadIdx.x; k < (int)(sizeof(FftPlanDev) / 4); k += blockDim.x)
        ((int *)sp)[k] = ((const int *)gp)[k];
    for (int k = threadIdx.x; k < ntab; k += blockDim.x) st[k] = gtab[gp->tab0 + k];
    for (int k = threadIdx.x; k < n; k += blockDim.x) stw[k] = gtw[gp->tw0 + k];
    ctx.p = sp;
    ctx.tab = st;
    ctx.tw = stw;
    return (unsigned char *)stw + align16(n * sizeof(float2));
}

// Full forward FFT of L lines of length n held in a (line stride in_ss); b is scratch.  The
// last pass is stored in the mode given with stride out_ds (MODE 1: the transposed row
// stride); the stages between keep the spread layout.  Returns the buffer holding the
// result; CONJ_LAST conjugates the final output (second half of an inverse transform).
template <int LAST_MODE, bool CONJ_LAST, bool WIDE = false>
__device__ float2 *fft_lines(const FftCtx &c, float2 *a, float2 *b, float *rdst, int L, int keep, int in_ss,
                             int out_ds)
{
    const FftPlanDev &p = *c.p;
    float2 *src = a, *dst = b;
    const int n = p.n, nst = p.nst;
    for (int s = 0; s < nst; ++s) {
        const int2 *t = c.tab + p.off[s];
        if (s + 1 < nst) {
            if (s == 0)
                fft_pass<0, false, false, true, WIDE>(p.rad[s], src, dst, nullptr, L, in_ss, n, 0, p.ns[s], p.nb[s],
                                                p.magic[s], t, c.tw);
            else
                fft_pass<0, false, true, true, WIDE>(p.rad[s], src, dst, nullptr, L, n, n, 0, p.ns[s], p.nb[s], p.magic[s],
                                               t, c.tw);
        } else if (s == 0) {
            fft_pass<LAST_MODE, CONJ_LAST, false, false, WIDE>(p.rad[s], src, dst, rdst, L, in_ss, out_ds, keep, p.ns[s],
                                                         p.nb[s], p.magic[s], t, c.tw);
        } else {
            fft_pass<LAST_MODE, CONJ_LAST, true, false, WIDE>(p.rad[s], src, dst, rdst, L, n, out_ds, keep, p.ns[s],
                                                        p.nb[s], p.magic[s], t, c.tw);
        }
        float2 *x = src; src = dst; dst = x;
    }
    return src;
}

// float2 slots of each of the two plane buffers of the FP32 plane kernels: the packed rows
// (ceil(n2/2) lines of n1), the half spectrum (n1/2+1 lines of n2, stored with the odd row
// stride n2|1 after the forward x pass), the transposed inverse y output (n2 rows of stride
// (n1/2+1)|1), and either kind in the spread layout of the stages between; even, so the
// buffers after it stay 16-byte aligned
__host__ __device__ __forceinline__ int plane_buf_elems(int n1, int n2)
{
    const int n1h = n1 / 2 + 1, a = ((n2 + 1) / 2) * n1, b = n1h * n2;
    int m = swz_elems(a > b ? a : b);
    m = m > n1h * (n2 | 1) ? m : n1h * (n2 | 1);
    m = m > n2 * (n1h | 1) ? m : n2 * (n1h | 1);
    return (m + 1) & ~1;
}

// float2 slots of each zconv buffer: NB_TKF lines of n3 at the odd stride n3|1 or spread
__host__ __device__ __forceinline__ int zconv_buf_elems(int n3)
{
    const int a = swz_elems(NB_TKF * n3), b = NB_TKF * (n3 | 1);
    return ((a > b ? a : b) + 1) & ~1;
}

__global__ void __launch_bounds__(256) k_plane_fwd_f(const PlaneWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                     const FftPlanDev *__restrict__ plans, const int *__restrict__ rep_plan,
                                                     const float2 *__restrict__ tw, const int2 *__restrict__ tab,
                                                     const int *__restrict__ zstart, const int *__restrict__ zatoms,
                                                     const float4 *__restrict__ fr, float2 *__restrict__ grid)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const PlaneWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n1h = R.n1h, n2p = (n2 + 1) >> 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    float2 *B0 = (float2 *)smem, *B1 = B0 + plane_buf_elems(n1, n2);
    int *acc = (int *)B0;                        // the int32 plane lives in B0 until it is packed
    FftCtx c1, c2;
    unsigned char *ctx = (unsigned char *)(B1 + plane_buf_elems(n1, n2));
    ctx = fft_ctx_load(ctx, plans + rep_plan[3 * w.rep], tab, tw, c1);
    fft_ctx_load(ctx, plans + rep_plan[3 * w.rep + 1], tab, tw, c2);
    for (int k = threadIdx.x; k < n1 * n2; k += blockDim.x) acc[k] = 0;
    __syncthreads();
    spread_plane<float>(R, w.z, zstart, zatoms, fr, acc, R.spread216);
    __syncthreads();
    // x transform of real rows two at a time: line p carries row 2p as its real part and
    // row 2p+1 as its imaginary part
    const float inv = R.spread_inv;
    for (int p = warp; p < n2p; p += nwarp)
        for (int x = lane; x < n1; x += 32) {
            const float re = Acc<float>::get(acc[2 * p * n1 + x], inv);
            const float im = 2 * p + 1 < n2 ? Acc<float>::get(acc[(2 * p + 1) * n1 + x], inv) : 0.f;
            B1[p * n1 + x] = make_float2(re, im);
        }
    __syncthreads();
    float2 *Z = fft_lines<0, false>(c1, B1, B0, nullptr, n2p, 0, n1, n1);
    float2 *T = Z == B1 ? B0 : B1;
    // separate the two real transforms (X_2p = (Z_k + conj Z_-k)/2, X_2p+1 = -i (Z_k - conj Z_-k)/2)
    // and keep kx < n1h, transposed to [kx][y] lines of n2 at the odd row stride sT (the lanes'
    // stores then fall in distinct banks)
    const int sT = n2 | 1;
    for (int p = warp; p < n2p; p += nwarp)
        for (int k = lane; k < n1h; k += 32) {
            const float2 a = Z[p * n1 + k], b = Z[p * n1 + (k == 0 ? 0 : n1 - k)];
            T[k * sT + 2 * p] = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
            if (2 * p + 1 < n2) T[k * sT + 2 * p + 1] = make_float2(0.5f * (a.y + b.y), 0.5f * (b.x - a.x));
        }
    __syncthreads();
    // y: n1h lines of n2
    float2 *Y = fft_lines<0, false>(c2, T, Z, nullptr, n1h, 0, sT, n2);
    float2 *g = grid + R.g0 + (size_t)w.z * n1h * n2;
    for (int k = threadIdx.x; k < n1h * n2; k += blockDim.x) g[k] = Y[k];
}

__global__ void __launch_bounds__(256, 6) k_zconv_f(const ColWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                 const FftPlanDev *__restrict__ plans, const int *__restrict__ rep_plan,
                                                 const float2 *__restrict__ tw, const int2 *__restrict__ tab,
                                                 const float *__restrict__ etab_all, float2 *__restrict__ grid,
                                                 double *__restrict__ e_col)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[8];
    const ColWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3, n1h = R.n1h;
    const int tk = w.nky;
    const float *etab = etab_all + R.bsp0;
    float2 *A = (float2 *)smem, *B = A + zconv_buf_elems(n3);
    FftCtx c3;
    fft_ctx_load((unsigned char *)(B + zconv_buf_elems(n3)), plans + rep_plan[3 * w.rep + 2], tab, tw, c3);
    const int sA = n3 | 1;    // odd line stride of the columns as loaded and stored
    float2 *g = grid + R.g0 + (size_t)w.kx * n2 + w.ky0;
    const size_t zs = (size_t)n1h * n2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int kz = warp; kz < n3; kz += 8)
        if (lane < tk) A[lane * sA + kz] = g[kz * zs + lane];
    __syncthreads();
    float2 *F = fft_lines<0, false, true>(c3, A, B, nullptr, tk, 0, sA, n3);
    float2 *Fo = F == A ? B : A;
    const float wgt = (w.kx == 0 || 2 * w.kx == n1) ? 1.f : 2.f;
    // influence function exp(-pi^2 m^2 / alpha^2) / (pi V B(m) m^2): the exponential and the
    // B-spline moduli factor per dimension, so they come from a per-dimension table
    // etab[k] = exp(-pi^2 m_k^2 / (alpha^2 L^2)) / B(k) formed in FP64 (no approximate
    // exponential in the energy); m^2 = sum_d k_d^2 / L_d^2 from exact integer squares and
    // 1/L_d^2 as hi + lo, and the reciprocal of pi V m^2 to within an ulp (one Newton step on
    // the approximate reciprocal, its residual formed exactly by an FMA)
    const float pivol = R.pivolf;
    const int nf2 = (n2 + 1) / 2, nf3 = (n3 + 1) / 2;
    const float m1s = (float)(w.kx * w.kx), t1 = etab[w.kx];
    const float c2h = R.msq_c[2][0], c2l = R.msq_c[2][1];
    float en = 0.f;
    for (int c = warp; c < tk; c += 8) {
        const int ky = w.ky0 + c;
        const int m2 = ky < nf2 ? ky : ky - n2;
        const float m2s = (float)(m2 * m2);
        const float t12 = t1 * etab[n1 + ky];
        const float m12 = fmaf(m1s, R.msq_c[0][0], fmaf(m2s, R.msq_c[1][0], fmaf(m1s, R.msq_c[0][1], m2s * R.msq_c[1][1])));
        for (int kz = lane; kz < n3; kz += 32) {
            const int m3 = kz < nf3 ? kz : kz - n3;
            const float m3s = (float)(m3 * m3);
            const float msq = fmaf(m3s, c2h, fmaf(m3s, c2l, m12));
            const float den = pivol * msq;
            float rd = nb_rcp_approx(den);
            rd = fmaf(rd, fmaf(-den, rd, 1.f), rd);
            const float et = (w.kx == 0 && ky == 0 && kz == 0) ? 0.f : (t12 * etab[n1 + n2 + kz]) * rd;
            float2 v = F[c * n3 + kz];
            en += wgt * et * (v.x * v.x + v.y * v.y);
            F[c * n3 + kz] = make_float2(v.x * et, -v.y * et);    // conj: the inverse runs forward
        }
    }
    __syncthreads();
    float2 *I = fft_lines<0, true, true>(c3, F, Fo, nullptr, tk, 0, n3, sA);
    for (int kz = warp; kz < n3; kz += 8)
        if (lane < tk) g[kz * zs + lane] = I[lane * sA + kz];
    // fixed-order reduction: each thread's few terms in FP32, then FP64 across the warp and
    // over the 8 warp sums; pivol_corr and pme_qcorr remove the FP32 rounding of pi V and of the
    // spread charges from the sum
    double ed = (double)en;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ed += __shfl_down_sync(0xffffffffu, ed, o);
    if (lane == 0) red[warp] = ed;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int k = 0; k < 8; ++k) sum += red[k];
        e_col[blockIdx.x] = sum * (R.pivol_corr * R.pme_qcorr);
    }
}

// Reciprocal virial of the pressure analysis (ewald_receip.f:799-807, pressON): the z
// transform of k_zconv_f's columns, then per m the diagonal terms
// E(m) (1 - 2 (1 + pi^2 m^2 / alpha^2) m_a^2 / m^2) with E(m) = wgt * eterm * |S(m)|^2 as the
// energy sum forms it; three FP64 partial sums per column work item (fixed-order reduction)
__global__ void __launch_bounds__(256) k_press_zvir_f(const ColWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                      const FftPlanDev *__restrict__ plans,
                                                      const int *__restrict__ rep_plan, const float2 *__restrict__ tw,
                                                      const int2 *__restrict__ tab, const float *__restrict__ bsp_all,
                                                      const float2 *__restrict__ grid, double *__restrict__ v_col)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[3][8];
    const ColWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3, n1h = R.n1h;
    const int tk = w.nky;
    const float *bsp = bsp_all + R.bsp0;
    float2 *A = (float2 *)smem, *B = A + zconv_buf_elems(n3);
    FftCtx c3;
    fft_ctx_load((unsigned char *)(B + zconv_buf_elems(n3)), plans + rep_plan[3 * w.rep + 2], tab, tw, c3);
    const int sA = n3 | 1;
    const float2 *g = grid + R.g0 + (size_t)w.kx * n2 + w.ky0;
    const size_t zs = (size_t)n1h * n2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int kz = warp; kz < n3; kz += 8)
        if (lane < tk) A[lane * sA + kz] = g[kz * zs + lane];
    __syncthreads();
    const float2 *F = fft_lines<0, false, true>(c3, A, B, nullptr, tk, 0, sA, n3);
    const float wgt = (w.kx == 0 || 2 * w.kx == n1) ? 1.f : 2.f;
    const float fac2 = R.pme_fac2f, pivol = R.pivolf, fac = (float)R.pme_fac;
    const int nf2 = (n2 + 1) / 2, nf3 = (n3 + 1) / 2;
    const float iL0 = R.invL[0], iL1 = R.invL[1], iL2 = R.invL[2];
    const float mh1 = (float)w.kx * iL0, pb1 = pivol * bsp[w.kx];
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    for (int c = warp; c < tk; c += 8) {
        const int ky = w.ky0 + c;
        const float mh2 = (float)(ky < nf2 ? ky : ky - n2) * iL1;
        const float pb12 = pb1 * bsp[n1 + ky], m12 = mh1 * mh1 + mh2 * mh2;
        for (int kz = lane; kz < n3; kz += 32) {
            if (w.kx == 0 && ky == 0 && kz == 0) continue;
            const float mh3 = (float)(kz < nf3 ? kz : kz - n3) * iL2;
            const float msq = fmaf(mh3, mh3, m12);
            const float et = nb_ex2_approx(-fac2 * msq) * nb_rcp_approx(pb12 * bsp[n1 + n2 + kz] * msq);
            const float2 v = F[c * n3 + kz];
            const float e = wgt * et * (v.x * v.x + v.y * v.y), b = 2.f * (1.f + fac * msq) / msq;
            v0 += e * (1.f - b * mh1 * mh1);
            v1 += e * (1.f - b * mh2 * mh2);
            v2 += e * (1.f - b * mh3 * mh3);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, o);
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
        v2 += __shfl_down_sync(0xffffffffu, v2, o);
    }
    if (lane == 0) { red[0][warp] = v0; red[1][warp] = v1; red[2][warp] = v2; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double sum = 0.0;
        for (int k = 0; k < 8; ++k) sum += red[threadIdx.x][k];
        v_col[3 * (size_t)blockIdx.x + threadIdx.x] = sum;
    }
}

// inverse y and x transforms of plane z; the real potential plane (n1 x n2 floats) is stored
// over the plane's own complex storage, which this block alone reads, for k_pme_gather_f
__global__ void __launch_bounds__(256) k_plane_inv_f(const PlaneWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                     const FftPlanDev *__restrict__ plans, const int *__restrict__ rep_plan,
                                                     const float2 *__restrict__ tw, const int2 *__restrict__ tab,
                                                     float2 *__restrict__ grid)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const PlaneWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n1h = R.n1h, n2p = (n2 + 1) >> 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    float2 *B0 = (float2 *)smem, *B1 = B0 + plane_buf_elems(n1, n2);
    FftCtx c1, c2;
    unsigned char *ctx = (unsigned char *)(B1 + plane_buf_elems(n1, n2));
    ctx = fft_ctx_load(ctx, plans + rep_plan[3 * w.rep], tab, tw, c1);
    fft_ctx_load(ctx, plans + rep_plan[3 * w.rep + 1], tab, tw, c2);
    float2 *g = grid + R.g0 + (size_t)w.z * n1h * n2;
    // [kx][ky] lines of n2, conjugated (inverse through the forward transform)
    for (int k = threadIdx.x; k < n1h * n2; k += blockDim.x) B0[k] = cconj(g[k]);
    __syncthreads();
    // y: n1h lines; last pass conjugates back and stores transposed to H[ky][kx] at the odd
    // row stride hs
    const int hs = n1h | 1;
    fft_lines<1, true>(c2, B0, B1, nullptr, n1h, n2, n2, hs);
    // which buffer got the transposed result depends on the pass count
    float2 *H = (c2.p->nst & 1) ? B1 : B0;
    float2 *Zc = H == B0 ? B1 : B0;
    // x inverse of two real rows at a time: Z = H_2p + i H_2p+1 over the full Hermitian line of
    // n1, conjugated so the forward transform inverts it; row 2p = Re, row 2p+1 = -Im of the result
    for (int p = warp; p < n2p; p += nwarp)
        for (int k = lane; k < n1; k += 32) {
            const bool lo = k < n1h;
            const int kk = lo ? k : n1 - k;
            float2 a = H[2 * p * hs + kk];
            float2 b = 2 * p + 1 < n2 ? H[(2 * p + 1) * hs + kk] : make_float2(0.f, 0.f);
            if (!lo) { a = cconj(a); b = cconj(b); }
            Zc[p * n1 + k] = make_float2(a.x - b.y, -(a.y + b.x));
        }
    __syncthreads();
    const float2 *W = fft_lines<0, false>(c1, Zc, H, nullptr, n2p, 0, n1, n1);
    // the real potential plane over the plane's own complex storage (this block alone reads it)
    float *gr = (float *)g;
    for (int p = warp; p < n2p; p += nwarp)
        for (int x = lane; x < n1; x += 32) {
            const float2 v = W[p * n1 + x];
            gr[2 * p * n1 + x] = v.x;
            if (2 * p + 1 < n2) gr[(2 * p + 1) * n1 + x] = -v.y;
        }
}

// PME gradient of each site from the real potential grid (grad_sum,
// ewald_receip.f:815-970): order-4 weights and derivatives once per site, the 4x4x4 stencil
// read from the grid planes k_plane_inv_f left in place; result (x, y, z) per site, to be
// scaled by q * fc * n_d / L_d in the finalize
__global__ void __launch_bounds__(256, 4) k_pme_gather_f(int nsite, const int *__restrict__ site_rep,
                                                      const RepDev *__restrict__ reps, const float4 *__restrict__ fr,
                                                      const float2 *__restrict__ grid, float4 *__restrict__ part)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    const float4 f = fr[s];
    if (f.w == 0.f) { part[s] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    const RepDev &R = reps[site_rep[s]];
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3;
    const size_t zs = (size_t)R.n1h * n2 * 2;    // floats per plane
    const float *Q = (const float *)(grid + R.g0);
    int i1, i2, i3;
    float w1, w2, w3;
    pme_fr_split(f.x, i1, w1);
    pme_fr_split(f.y, i2, w2);
    pme_fr_split(f.z, i3, w3);
    float th1[4], dt1[4], th2[4], dt2[4], th3[4], dt3[4];
    bsp4_th<float>(w1, th1); bsp4_dth<float>(w1, dt1);
    bsp4_th<float>(w2, th2); bsp4_dth<float>(w2, dt2);
    bsp4_th<float>(w3, th3); bsp4_dth<float>(w3, dt3);
    int xs[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) xs[t] = pme_wrap(i1 - 3 + t, n1);
    // without an x wrap the four stencil points of a row are contiguous: two aligned float4
    // loads hold them, one when they start 16-byte aligned (the grid allocation ends 16 bytes
    // past its last plane for the second).
    // fr1 can round to n1 itself (index n1 wraps to 0), which takes the wrapped path.
    const bool contig = i1 >= 3 && i1 < n1;
    float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
    for (int t3 = 0; t3 < 4; ++t3) {
        const float *P = Q + pme_wrap(i3 - 3 + t3, n3) * zs;
        float hx = 0.f, hy = 0.f, hz = 0.f;
#pragma unroll
        for (int t2 = 0; t2 < 4; ++t2) {
            const float *row = P + pme_wrap(i2 - 3 + t2, n2) * n1;
            float q4[4];
            if (contig) {
                const uintptr_t a = (uintptr_t)(row + i1 - 3);
                const float4 *p4 = (const float4 *)(a & ~(uintptr_t)15);
                const int sh = (int)((a >> 2) & 3);
                const float4 c0 = __ldg(p4);
                const float4 c1 = sh != 0 ? __ldg(p4 + 1) : c0;     // an aligned row needs one load
                q4[0] = sh == 0 ? c0.x : (sh == 1 ? c0.y : (sh == 2 ? c0.z : c0.w));
                q4[1] = sh == 0 ? c0.y : (sh == 1 ? c0.z : (sh == 2 ? c0.w : c1.x));
                q4[2] = sh == 0 ? c0.z : (sh == 1 ? c0.w : (sh == 2 ? c1.x : c1.y));
                q4[3] = sh == 0 ? c0.w : (sh == 1 ? c1.x : (sh == 2 ? c1.y : c1.z));
            } else {
#pragma unroll
                for (int t1 = 0; t1 < 4; ++t1) q4[t1] = row[xs[t1]];
            }
            float sx = 0.f, sy = 0.f;
#pragma unroll
            for (int t1 = 0; t1 < 4; ++t1) {
                const float q = q4[t1];
                sx = fmaf(q, dt1[t1], sx);
                sy = fmaf(q, th1[t1], sy);
            }
            hx = fmaf(sx, th2[t2], hx);
            hy = fmaf(sy, dt2[t2], hy);
            hz = fmaf(sy, th2[t2], hz);
        }
        gx = fmaf(hx, th3[t3], gx);
        gy = fmaf(hy, th3[t3], gy);
        gz = fmaf(hz, dt3[t3], gz);
    }
    part[s] = make_float4(gx, gy, gz, 0.f);
}

// =================================================================================
// FP64 (plain) path: one warp per line, same grid layout [z][kx][ky]

template <typename C>
__device__ C *warp_fft(C *x, C *y, const FftPlanDev &p, const C *__restrict__ tw, int lane)
{
    int n = p.n, Ns = 1;
    for (int st = 0; st < p.nst; ++st) {
        int R = p.rad[st], nb = n / R, stride = n / (Ns * R);
        for (int j = lane; j < nb; j += 32) {
            C v[5];
            int jm = j % Ns;
            for (int r = 0; r < R; ++r) v[r] = x[j + r * nb];
            int tstep = jm * stride;
            for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * tstep]);
            if (R == 4) bfly4(v);
            else if (R == 2) bfly2(v);
            else if (R == 3) bfly3(v);
            else bfly5(v);
            int idxD = (j / Ns) * Ns * R + jm;
            for (int r = 0; r < R; ++r) y[idxD + r * Ns] = v[r];
        }
        __syncwarp();
        C *t = x; x = y; y = t;
        Ns *= R;
    }
    return x;
}

#define NB_TK 16

template <typename T>
__global__ void __launch_bounds__(256) k_plane_fwd(const PlaneWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                   const FftPlanDev *__restrict__ plans, const int *__restrict__ rep_plan,
                                                   const void *tw_v, const int *__restrict__ zstart,
                                                   const int *__restrict__ zatoms, const void *fr_v, void *grid_v)
{
    typedef typename cplx<T>::type C;
    typedef typename Acc<T>::type A;
    extern __shared__ __align__(16) unsigned char smem[];
    PlaneWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n1h = R.n1h, pitch = n1h | 1;
    const FftPlanDev p1 = plans[rep_plan[3 * w.rep]], p2 = plans[rep_plan[3 * w.rep + 1]];
    const C *tw = (const C *)tw_v;
    A *acc = (A *)smem;
    C *P = (C *)(smem + align16(sizeof(A) * n1 * n2));
    C *scr = P + n2 * pitch;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int k = threadIdx.x; k < n1 * n2; k += blockDim.x) acc[k] = 0;
    __syncthreads();
    spread_plane<T>(R, w.z, zstart, zatoms, (const typename vec4<T>::type *)fr_v, acc, (T)1);
    __syncthreads();
    C *x = scr + warp * 2 * NB_MAX_FFT, *y = x + NB_MAX_FFT;
    for (int j = warp; j < n2; j += nwarp) {
        for (int i = lane; i < n1; i += 32) { x[i].x = Acc<T>::get(acc[j * n1 + i], (T)1); x[i].y = 0; }
        __syncwarp();
        C *res = warp_fft<C>(x, y, p1, tw + p1.tw0, lane);
        for (int k = lane; k < n1h; k += 32) P[j * pitch + k] = res[k];
        __syncwarp();
    }
    __syncthreads();
    for (int k = warp; k < n1h; k += nwarp) {
        for (int j = lane; j < n2; j += 32) x[j] = P[j * pitch + k];
        __syncwarp();
        C *res = warp_fft<C>(x, y, p2, tw + p2.tw0, lane);
        for (int j = lane; j < n2; j += 32) P[j * pitch + k] = res[j];
        __syncwarp();
    }
    __syncthreads();
    C *g = (C *)grid_v + R.g0 + (size_t)w.z * n2 * n1h;
    for (int idx = threadIdx.x; idx < n2 * n1h; idx += blockDim.x) {
        int kx = idx / n2, ky = idx - kx * n2;
        g[idx] = P[ky * pitch + kx];
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_zconv(const ColWork *__restrict__ work, const RepDev *__restrict__ reps,
                                               const FftPlanDev *__restrict__ plans, const int *__restrict__ rep_plan,
                                               const void *tw_v, const void *bsp_v, void *grid_v,
                                               double *__restrict__ e_col)
{
    typedef typename cplx<T>::type C;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[256];
    ColWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3, n1h = R.n1h;
    const int tk = w.nky;
    const int n3p = n3 | 1;
    const FftPlanDev p3 = plans[rep_plan[3 * w.rep + 2]];
    const C *tw = (const C *)tw_v;
    const T *bsp = (const T *)bsp_v + R.bsp0;
    C *tile = (C *)smem;
    C *scr = tile + NB_TK * n3p;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    C *g = (C *)grid_v + R.g0 + (size_t)w.kx * n2 + w.ky0;
    const size_t zs = (size_t)n1h * n2;
    for (int idx = threadIdx.x; idx < tk * n3; idx += blockDim.x) {
        int kz = idx / tk, c = idx - kz * tk;
        tile[c * n3p + kz] = g[kz * zs + c];
    }
    __syncthreads();
    double en = 0;
    C *x = scr + warp * 2 * NB_MAX_FFT, *y = x + NB_MAX_FFT;
    const T wgt = (w.kx == 0 || (2 * w.kx == n1)) ? (T)1 : (T)2;
    for (int c = warp; c < tk; c += nwarp) {
        const int ky = w.ky0 + c;
        for (int kz = lane; kz < n3; kz += 32) x[kz] = tile[c * n3p + kz];
        __syncwarp();
        C *res = warp_fft<C>(x, y, p3, tw + p3.tw0, lane);
        for (int kz = lane; kz < n3; kz += 32) {
            T et = eterm_of<T>(R, bsp, w.kx, ky, kz);
            C v = res[kz];
            en += (double)(wgt * et * (v.x * v.x + v.y * v.y));
            v.x *= et;
            v.y *= et;
            res[kz] = cconj(v);
        }
        __syncwarp();
        C *other = (res == x) ? y : x;
        C *res2 = warp_fft<C>(res, other, p3, tw + p3.tw0, lane);
        for (int kz = lane; kz < n3; kz += 32) tile[c * n3p + kz] = cconj(res2[kz]);
        __syncwarp();
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < tk * n3; idx += blockDim.x) {
        int kz = idx / tk, c = idx - kz * tk;
        g[kz * zs + c] = tile[c * n3p + kz];
    }
    red[threadIdx.x] = en;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) e_col[blockIdx.x] = red[0];
}

// reciprocal virial of the pressure analysis on the plain path: the z transform of k_zconv's
// columns (one warp per line), then per m the diagonal terms
// E(m) (1 - 2 (1 + pi^2 m^2 / alpha^2) m_a^2 / m^2) (ewald_receip.f:799-807), E(m) as the
// energy sum forms it; three FP64 sums per column work item
template <typename T>
__global__ void __launch_bounds__(256) k_press_zvir(const ColWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                    const FftPlanDev *__restrict__ plans,
                                                    const int *__restrict__ rep_plan, const void *tw_v,
                                                    const void *bsp_v, const void *grid_v, double *__restrict__ v_col)
{
    typedef typename cplx<T>::type C;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[3][256];
    const ColWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n3 = R.n3, n1h = R.n1h;
    const int tk = w.nky;
    const int n3p = n3 | 1;
    const FftPlanDev p3 = plans[rep_plan[3 * w.rep + 2]];
    const C *tw = (const C *)tw_v;
    const T *bsp = (const T *)bsp_v + R.bsp0;
    C *tile = (C *)smem;
    C *scr = tile + NB_TK * n3p;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const C *g = (const C *)grid_v + R.g0 + (size_t)w.kx * n2 + w.ky0;
    const size_t zs = (size_t)n1h * n2;
    for (int idx = threadIdx.x; idx < tk * n3; idx += blockDim.x) {
        const int kz = idx / tk, c = idx - kz * tk;
        tile[c * n3p + kz] = g[kz * zs + c];
    }
    __syncthreads();
    double v[3] = {0.0, 0.0, 0.0};
    C *x = scr + warp * 2 * NB_MAX_FFT, *y = x + NB_MAX_FFT;
    const double wgt = (w.kx == 0 || (2 * w.kx == n1)) ? 1.0 : 2.0;
    const int nf2 = (n2 + 1) / 2, nf3 = (n3 + 1) / 2;
    for (int c = warp; c < tk; c += nwarp) {
        const int ky = w.ky0 + c;
        for (int kz = lane; kz < n3; kz += 32) x[kz] = tile[c * n3p + kz];
        __syncwarp();
        const C *res = warp_fft<C>(x, y, p3, tw + p3.tw0, lane);
        for (int kz = lane; kz < n3; kz += 32) {
            if (w.kx == 0 && ky == 0 && kz == 0) continue;
            const double mh[3] = {(double)w.kx * R.invLd[0], (double)(ky < nf2 ? ky : ky - n2) * R.invLd[1],
                                  (double)(kz < nf3 ? kz : kz - n3) * R.invLd[2]};
            const double msq = mh[0] * mh[0] + mh[1] * mh[1] + mh[2] * mh[2];
            const double et = (double)eterm_of<T>(R, bsp, w.kx, ky, kz);
            const C q = res[kz];
            const double e = wgt * et * ((double)q.x * q.x + (double)q.y * q.y), b = 2.0 * (1.0 + R.pme_fac * msq) / msq;
#pragma unroll
            for (int d = 0; d < 3; ++d) v[d] += e * (1.0 - b * mh[d] * mh[d]);
        }
        __syncwarp();
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) red[d][threadIdx.x] = v[d];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
#pragma unroll
            for (int d = 0; d < 3; ++d) red[d][threadIdx.x] += red[d][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 3) v_col[3 * (size_t)blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

template <typename T>
__global__ void __launch_bounds__(256) k_plane_inv(const PlaneWork *__restrict__ work, const RepDev *__restrict__ reps,
                                                   const FftPlanDev *__restrict__ plans, const int *__restrict__ rep_plan,
                                                   const void *tw_v, const int *__restrict__ zstart,
                                                   const int *__restrict__ zatoms, const void *fr_v,
                                                   const void *grid_v, T *__restrict__ part, int pot)
{
    typedef typename cplx<T>::type C;
    extern __shared__ __align__(16) unsigned char smem[];
    PlaneWork w = work[blockIdx.x];
    const RepDev &R = reps[w.rep];
    const int n1 = R.n1, n2 = R.n2, n1h = R.n1h, pitch = n1h | 1;
    const FftPlanDev p1 = plans[rep_plan[3 * w.rep]], p2 = plans[rep_plan[3 * w.rep + 1]];
    const C *tw = (const C *)tw_v;
    T *Rp = (T *)smem;
    C *P = (C *)(smem + align16(sizeof(T) * n1 * n2));
    C *scr = P + n2 * pitch;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const C *g = (const C *)grid_v + R.g0 + (size_t)w.z * n2 * n1h;
    for (int idx = threadIdx.x; idx < n2 * n1h; idx += blockDim.x) {
        int kx = idx / n2, ky = idx - kx * n2;
        P[ky * pitch + kx] = g[idx];
    }
    __syncthreads();
    C *x = scr + warp * 2 * NB_MAX_FFT, *y = x + NB_MAX_FFT;
    for (int k = warp; k < n1h; k += nwarp) {
        for (int j = lane; j < n2; j += 32) x[j] = cconj(P[j * pitch + k]);
        __syncwarp();
        C *res = warp_fft<C>(x, y, p2, tw + p2.tw0, lane);
        for (int j = lane; j < n2; j += 32) P[j * pitch + k] = cconj(res[j]);
        __syncwarp();
    }
    __syncthreads();
    for (int j = warp; j < n2; j += nwarp) {
        for (int i = lane; i < n1; i += 32) {
            C v = i < n1h ? P[j * pitch + i] : cconj(P[j * pitch + (n1 - i)]);
            x[i] = cconj(v);
        }
        __syncwarp();
        C *res = warp_fft<C>(x, y, p1, tw + p1.tw0, lane);
        for (int i = lane; i < n1; i += 32) Rp[j * n1 + i] = res[i].x;
        __syncwarp();
    }
    __syncthreads();
    gather_plane<T>(R, w.z, zstart, zatoms, (const typename vec4<T>::type *)fr_v, Rp, part, pot != 0);
}

// ---------------------------------------------------------------------------------
// launch sequence (both precisions)

template <typename T>
void pme_t(NbCtx *c)
{
    cudaStream_t s = c->stream;
    const int B = 256;
    if (c->timing) cudaEventRecord(c->ev[6], s);
    cudaMemsetAsync(c->d_zcount, 0, sizeof(int) * (c->nzbin + 1), s);
    k_pme_bin<T><<<(int)((c->nsite + B - 1) / B), B, 0, s>>>((int)c->nsite, c->d_site_rep, c->d_reps, c->d_pos,
                                                            c->d_site_q, c->d_fr, c->d_zcount, c->d_zslot);
    nb_exclusive_scan(c, c->d_zcount, c->d_zstart, c->nzbin, nullptr);
    k_pme_scatter<<<(int)((c->nsite + B - 1) / B), B, 0, s>>>((int)c->nsite, c->d_site_rep, c->d_reps, c->d_fr,
                                                             sizeof(T) == 8, c->d_zstart, c->d_zslot, c->d_zatoms);
    const int np = (int)c->planes.size(), nc = (int)c->cols.size();
    if (sizeof(T) == 4) {
        k_plane_fwd_f<<<np, 256, c->smem_plane_fwd, s>>>(c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan,
                                                           (const float2 *)c->d_tw, c->d_tab, c->d_zstart,
                                                           c->d_zatoms, (const float4 *)c->d_fr, (float2 *)c->d_grid);
        if (c->timing) cudaEventRecord(c->ev[7], s);
        k_zconv_f<<<nc, 256, c->smem_zconv, s>>>(c->d_cols, c->d_reps, c->d_plans, c->d_rep_plan,
                                                  (const float2 *)c->d_tw, c->d_tab, c->d_etab,
                                                  (float2 *)c->d_grid, c->d_e_col);
        if (c->timing) cudaEventRecord(c->ev[8], s);
        k_plane_inv_f<<<np, 256, c->smem_plane_inv, s>>>(c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan,
                                                           (const float2 *)c->d_tw, c->d_tab, (float2 *)c->d_grid);
        k_pme_gather_f<<<(int)((c->nsite + 255) / 256), 256, 0, s>>>(
            (int)c->nsite, c->d_site_rep, c->d_reps, (const float4 *)c->d_fr, (const float2 *)c->d_grid,
            (float4 *)c->d_part);
        c->launches++;
    } else {
        k_plane_fwd<T><<<np, 256, c->smem_plane_fwd, s>>>(c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan, c->d_tw,
                                                          c->d_zstart, c->d_zatoms, c->d_fr, c->d_grid);
        if (c->timing) cudaEventRecord(c->ev[7], s);
        k_zconv<T><<<nc, 256, c->smem_zconv, s>>>(c->d_cols, c->d_reps, c->d_plans, c->d_rep_plan, c->d_tw,
                                                   c->d_bsp, c->d_grid, c->d_e_col);
        if (c->timing) cudaEventRecord(c->ev[8], s);
        k_plane_inv<T><<<np, 256, c->smem_plane_inv, s>>>(c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan, c->d_tw,
                                                          c->d_zstart, c->d_zatoms, c->d_fr, c->d_grid,
                                                          (T *)c->d_part, 0);
    }
    if (c->timing) cudaEventRecord(c->ev[9], s);
    c->launches += 6;
}

// radix plan and Stockham tables; returns 0 if n is not 2/3/5-smooth or too long.  Narrow
// plans (the plane kernels and the FP64 one-warp-per-line transform) take 4s first, then 2, 3,
// 5.  Wide plans (the FP32 z columns) also have the composite codelets 6, 8, 9, 10 and take
// the fewest passes (a line of up to 100 points in two), larger radices first on ties.  tab
// receives (twiddle step, destination index) per butterfly.
// fewest factors of m from the wide radix set, at most `left` of them (-1: none)
int wide_factors(int m, int left, int *out)
{
    static const int R[8] = {10, 9, 8, 6, 5, 4, 3, 2};
    if (m == 1) return 0;
    if (left == 0) return -1;
    int best = -1, tmp[8];
    for (int k = 0; k < 8; ++k) {
        if (m % R[k]) continue;
        const int f = wide_factors(m / R[k], best < 0 ? left - 1 : best - 2, tmp);
        if (f < 0) continue;
        best = f + 1;
        out[0] = R[k];
        for (int q = 0; q < f; ++q) out[1 + q] = tmp[q];
        if (best == 1) break;
    }
    return best;
}

int make_plan(int n, FftPlanDev *p, std::vector<int2> *tab, bool wide)
{
    memset(p, 0, sizeof(*p));
    p->n = n;
    int m = n, k = 0;
    if (n < 2 || n > NB_MAX_FFT) return 0;
    if (wide) {
        k = wide_factors(n, 8, p->rad);
        if (k < 0) return 0;
        m = 1;
    } else {
        while (m % 4 == 0) { p->rad[k++] = 4; m /= 4; }
        while (m % 2 == 0) { p->rad[k++] = 2; m /= 2; }
        while (m % 3 == 0) { p->rad[k++] = 3; m /= 3; }
        while (m % 5 == 0) { p->rad[k++] = 5; m /= 5; }
    }
    if (m != 1 || k > 8) return 0;
    p->nst = k;
    int Ns = 1, off = 0;
    for (int s = 0; s < k; ++s) {
        int R = p->rad[s], nb = n / R, stride = n / (Ns * R);
        p->ns[s] = Ns;
        p->nb[s] = nb;
        p->off[s] = off;
        p->magic[s] = nb > 1 ? 0xFFFFFFFFu / (unsigned)nb + 1u : 0u;
        if (tab) {
            for (int j = 0; j < nb; ++j) {
                int jm = j % Ns;
                tab->push_back(make_int2(jm * stride, (j / Ns) * Ns * R + jm));
            }
        }
        off += nb;
        Ns *= R;
    }
    return 1;
}

size_t fft_ctx_bytes(int n, bool wide)
{
    FftPlanDev p;
    if (!make_plan(n, &p, nullptr, wide)) return 0;
    size_t ntab = (size_t)p.off[p.nst - 1] + p.nb[p.nst - 1];
    return align16(sizeof(FftPlanDev)) + align16(ntab * sizeof(int2)) + align16(n * sizeof(float2));
}

template <typename T>
size_t plane_fwd_smem(int n1, int n2)
{
    if (sizeof(T) == 4) return (size_t)2 * plane_buf_elems(n1, n2) * sizeof(float2) + fft_ctx_bytes(n1, false) + fft_ctx_bytes(n2, false);
    typedef typename cplx<T>::type C;
    size_t acc = (sizeof(typename Acc<T>::type) * n1 * n2 + 15) & ~(size_t)15;
    return acc + sizeof(C) * n2 * ((n1 / 2 + 1) | 1) + sizeof(C) * 8 * 2 * NB_MAX_FFT;
}
template <typename T>
size_t plane_inv_smem(int n1, int n2)
{
    if (sizeof(T) == 4) return (size_t)2 * plane_buf_elems(n1, n2) * sizeof(float2) + fft_ctx_bytes(n1, false) + fft_ctx_bytes(n2, false);
    typedef typename cplx<T>::type C;
    size_t r = (sizeof(T) * n1 * n2 + 15) & ~(size_t)15;
    return r + sizeof(C) * n2 * ((n1 / 2 + 1) | 1) + sizeof(C) * 8 * 2 * NB_MAX_FFT;
}
template <typename T>
size_t zconv_smem(int n3)
{
    if (sizeof(T) == 4) return (size_t)2 * zconv_buf_elems(n3) * sizeof(float2) + fft_ctx_bytes(n3, true);
    typedef typename cplx<T>::type C;
    return sizeof(C) * NB_TK * (n3 | 1) + sizeof(C) * 8 * 2 * NB_MAX_FFT;
}
template <typename T> int col_tile() { return sizeof(T) == 4 ? NB_TKF : NB_TK; }

// the z-column work items of one kx: the n2 columns in ceil(n2 / tile) runs of equal length
// (within one), so no block of the column kernels works on a short remainder alone (n2 = 36
// gives two runs of 18, not 32 and 4: every Stockham pass of a run then fits one sweep of the
// block's threads)
void push_col_runs(std::vector<ColWork> &cols, int rep, int kx, int n2, int tile)
{
    const int nrun = (n2 + tile - 1) / tile, base = n2 / nrun, extra = n2 % nrun;
    int ky0 = 0;
    for (int k = 0; k < nrun; ++k) {
        const int len = base + (k < extra ? 1 : 0);
        cols.push_back(ColWork{rep, kx, ky0, len});
        ky0 += len;
    }
}

// raise a kernel's dynamic shared-memory limit to at least `bytes` (never lower it)
template <typename K>
cudaError_t raise_smem_limit(K *kernel, size_t bytes)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T>
cudaError_t raise_pme_limits(size_t sf, size_t sz, size_t si)
{
    cudaError_t e;
    if (sizeof(T) == 4) {
        if ((e = raise_smem_limit(k_plane_fwd_f, sf)) != cudaSuccess) return e;
        if ((e = raise_smem_limit(k_zconv_f, sz)) != cudaSuccess) return e;
        if ((e = raise_smem_limit(k_press_zvir_f, sz)) != cudaSuccess) return e;
        return raise_smem_limit(k_plane_inv_f, si);
    }
    if ((e = raise_smem_limit(k_plane_fwd<T>, sf)) != cudaSuccess) return e;
    if ((e = raise_smem_limit(k_zconv<T>, sz)) != cudaSuccess) return e;
    if ((e = raise_smem_limit(k_press_zvir<T>, sz)) != cudaSuccess) return e;
    return raise_smem_limit(k_plane_inv<T>, si);
}

template <typename T>
int configure_t(NbCtx *c)
{
    typedef typename cplx<T>::type C;
    c->plans.clear();
    c->rep_plan.assign(3 * c->nrep, 0);
    std::vector<double> twr, twi;
    std::vector<int2> tab;
    std::vector<char> wide_of;     // per plan: wide radix set (the FP32 z columns)
    for (int r = 0; r < c->nrep; ++r) {
        int ns[3] = {c->rd[r].n1, c->rd[r].n2, c->rd[r].n3};
        for (int d = 0; d < 3; ++d) {
            const bool wide = sizeof(T) == 4 && d == 2;
            int found = -1;
            for (size_t k = 0; k < c->plans.size(); ++k)
                if (c->plans[k].n == ns[d] && (bool)wide_of[k] == wide) found = (int)k;
            if (found < 0) {
                FftPlanDev p;
                int tab0 = (int)tab.size();
                if (!make_plan(ns[d], &p, &tab, wide)) return MOIL_NB_ERR_GRID;
                p.tab0 = tab0;
                p.tw0 = (int)twr.size();
                for (int t = 0; t < ns[d]; ++t) {
                    double ang = -2.0 * M_PI * (double)t / (double)ns[d];
                    twr.push_back(cos(ang));
                    twi.push_back(sin(ang));
                }
                c->plans.push_back(p);
                wide_of.push_back(wide);
                found = (int)c->plans.size() - 1;
            }
            c->rep_plan[3 * r + d] = found;
        }
    }
    std::vector<C> tw(twr.size());
    for (size_t k = 0; k < twr.size(); ++k) { tw[k].x = (T)twr[k]; tw[k].y = (T)twi[k]; }
    NB_CUDA_OK(c, cudaMalloc(&c->d_plans, sizeof(FftPlanDev) * c->plans.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_plans, c->plans.data(), sizeof(FftPlanDev) * c->plans.size(), cudaMemcpyHostToDevice));
    NB_CUDA_OK(c, cudaMalloc(&c->d_rep_plan, sizeof(int) * c->rep_plan.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_rep_plan, c->rep_plan.data(), sizeof(int) * c->rep_plan.size(), cudaMemcpyHostToDevice));
    NB_CUDA_OK(c, cudaMalloc(&c->d_tw, sizeof(C) * tw.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_tw, tw.data(), sizeof(C) * tw.size(), cudaMemcpyHostToDevice));
    NB_CUDA_OK(c, cudaMalloc(&c->d_tab, sizeof(int2) * tab.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_tab, tab.data(), sizeof(int2) * tab.size(), cudaMemcpyHostToDevice));
    std::vector<T> bsp(c->bsp_h.size());
    for (size_t k = 0; k < bsp.size(); ++k) bsp[k] = (T)c->bsp_h[k];
    NB_CUDA_OK(c, cudaMalloc(&c->d_bsp, sizeof(T) * bsp.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_bsp, bsp.data(), sizeof(T) * bsp.size(), cudaMemcpyHostToDevice));
    if (sizeof(T) == 4) {
        std::vector<float> et(c->bsp_h.size());
        for (int r = 0; r < c->nrep; ++r) {
            const RepDev &R = c->rd[r];
            nb_pme_etab(R, c->bsp_h.data() + R.bsp0, et.data() + R.bsp0);
        }
        NB_CUDA_OK(c, cudaMalloc(&c->d_etab, sizeof(float) * et.size()));
        NB_CUDA_OK(c, cudaMemcpy(c->d_etab, et.data(), sizeof(float) * et.size(), cudaMemcpyHostToDevice));
    }
    // work lists: planes (replica, z) and z columns (replica, kx, ky run)
    c->planes.clear();
    c->cols.clear();
    c->col_begin.assign(c->nrep + 1, 0);
    size_t sf = 0, si = 0, sz = 0;
    const int tk = col_tile<T>();
    for (int r = 0; r < c->nrep; ++r) {
        const RepDev &R = c->rd[r];
        for (int z = 0; z < R.n3; ++z) c->planes.push_back(PlaneWork{r, z});
        c->col_begin[r] = (int)c->cols.size();
        for (int kx = 0; kx < R.n1h; ++kx)
            push_col_runs(c->cols, r, kx, R.n2, tk);
        sf = std::max(sf, plane_fwd_smem<T>(R.n1, R.n2));
        si = std::max(si, plane_inv_smem<T>(R.n1, R.n2));
        sz = std::max(sz, zconv_smem<T>(R.n3));
    }
    c->col_begin[c->nrep] = (int)c->cols.size();
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    if ((int)sf > dev_smem || (int)si > dev_smem || (int)sz > dev_smem) {
        c->err = "PME grid plane does not fit in shared memory";
        return MOIL_NB_ERR_GRID;
    }
    c->smem_plane_fwd = sf;
    c->smem_plane_inv = si;
    c->smem_zconv = sz;
    // the limit is per kernel, shared by every handle in the process: only ever raise it
    NB_CUDA_OK(c, raise_pme_limits<T>(sf, sz, si));
    NB_CUDA_OK(c, cudaMalloc(&c->d_planes, sizeof(PlaneWork) * c->planes.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_planes, c->planes.data(), sizeof(PlaneWork) * c->planes.size(), cudaMemcpyHostToDevice));
    NB_CUDA_OK(c, cudaMalloc(&c->d_cols, sizeof(ColWork) * c->cols.size()));
    NB_CUDA_OK(c, cudaMemcpy(c->d_cols, c->cols.data(), sizeof(ColWork) * c->cols.size(), cudaMemcpyHostToDevice));
    NB_CUDA_OK(c, cudaMalloc(&c->d_col_begin, sizeof(int) * (c->nrep + 1)));
    NB_CUDA_OK(c, cudaMemcpy(c->d_col_begin, c->col_begin.data(), sizeof(int) * (c->nrep + 1), cudaMemcpyHostToDevice));
    NB_CUDA_OK(c, cudaMalloc(&c->d_e_col, sizeof(double) * c->cols.size()));
    // two spare elements: the FP32 gather's second aligned float4 of a row may reach 16 bytes
    // past the last plane
    NB_CUDA_OK(c, cudaMalloc(&c->d_grid, sizeof(C) * (c->grid_elems + 2)));
    NB_CUDA_OK(c, cudaMalloc(&c->d_fr, sizeof(typename vec4<T>::type) * c->nsite));
    NB_CUDA_OK(c, cudaMalloc(&c->d_part, sizeof(T) * 12 * c->nsite));
    NB_CUDA_OK(c, cudaMemset(c->d_part, 0, sizeof(T) * 12 * c->nsite));
    return MOIL_NB_OK;
}

}  // namespace

void nb_launch_pme(NbCtx *c)
{
    if (c->precision == MOIL_NB_FP64) pme_t<double>(c);
    else pme_t<float>(c);
}

// pressure analysis: the charge planes of the evaluation's binning spread and transformed
// again into grid (a copy beside the handle's own grid, whose potential planes stay valid),
// and the reciprocal virial per column work item into v_col (mixed path)
void nb_launch_pme_virial(NbCtx *c, void *grid, double *v_col)
{
    cudaStream_t s = c->stream;
    const int np = (int)c->planes.size(), nc = (int)c->cols.size();
    if (c->precision == MOIL_NB_FP64) {
        k_plane_fwd<double><<<np, 256, c->smem_plane_fwd, s>>>(c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan,
                                                               c->d_tw, c->d_zstart, c->d_zatoms, c->d_fr, grid);
        k_press_zvir<double><<<nc, 256, c->smem_zconv, s>>>(c->d_cols, c->d_reps, c->d_plans, c->d_rep_plan, c->d_tw,
                                                            c->d_bsp, grid, v_col);
        return;
    }
    k_plane_fwd_f<<<np, 256, c->smem_plane_fwd, s>>>(c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan,
                                                       (const float2 *)c->d_tw, c->d_tab, c->d_zstart, c->d_zatoms,
                                                       (const float4 *)c->d_fr, (float2 *)grid);
    k_press_zvir_f<<<nc, 256, c->smem_zconv, s>>>(c->d_cols, c->d_reps, c->d_plans, c->d_rep_plan,
                                                   (const float2 *)c->d_tw, c->d_tab, (const float *)c->d_bsp,
                                                   (const float2 *)grid, v_col);
}

// parameter derivatives on the plain path: the potential share of every plane at each site
// (4 slots per site) from the convolved grid the evaluation left in place
void nb_launch_pme_potential(NbCtx *c, double *phi4)
{
    k_plane_inv<double><<<(int)c->planes.size(), 256, c->smem_plane_inv, c->stream>>>(
        c->d_planes, c->d_reps, c->d_plans, c->d_rep_plan, c->d_tw, c->d_zstart, c->d_zatoms, c->d_fr, c->d_grid,
        phi4, 1);
}

int nb_pme_configure(NbCtx *c)
{
    return c->precision == MOIL_NB_FP64 ? configure_t<double>(c) : configure_t<float>(c);
}

void nb_spread_scale(double qfc_max, RepDev *R)
{
    const int k = nb_spread_exp(qfc_max);
    R->spread_scale = (float)ldexp(1.0, k);
    R->spread_inv = (float)ldexp(1.0, -k);
    const double s216 = ldexp(1.0, k) / 216.0;
    R->spread216 = (float)s216;
    R->spread216_corr = s216 / (double)R->spread216;
}

void nb_pme_etab(const RepDev &R, const double *bsp, float *out)
{
    const int ns[3] = {R.n1, R.n2, R.n3};
    for (int d = 0, o = 0; d < 3; o += ns[d], ++d)
        for (int k = 0; k < ns[d]; ++k) {
            // MOIL's m folding (pot/ewald_receip.f:723-812): k > ceil(n/2) - 1 -> k - n
            const int m = k < (ns[d] + 1) / 2 ? k : k - ns[d];
            const double mh = m * R.invLd[d];
            out[o + k] = (float)(exp(-R.pme_fac * mh * mh) / bsp[o + k]);
        }
}

void nb_pme_fp32_consts(RepDev *R)
{
    const double fac2 = R->pme_fac * 1.4426950408889634;
    R->pme_fac2f = (float)fac2;
    R->fac2_lo = (float)(fac2 - (double)R->pme_fac2f);
    R->pivolf = (float)R->pivol;
    R->pivol_corr = (double)R->pivolf / R->pivol;
    for (int d = 0; d < 3; ++d) R->invL_lo[d] = (float)(R->invLd[d] - (double)R->invL[d]);
    for (int d = 0; d < 3; ++d) {
        const double c = R->invLd[d] * R->invLd[d];
        R->msq_c[d][0] = (float)c;
        R->msq_c[d][1] = (float)(c - (double)R->msq_c[d][0]);
    }
}

// ---------------------------------------------------------------------------------
// Allocation-free PME reciprocal sum (moil_nb_pme_noalloc).
//
// For callers that cannot allocate device memory: the same bin / spread+FFT / convolution /
// FFT+gather kernels as the handle path (FP32), with every scratch buffer carved out of one
// file-scope device array.  The array is sized for at most NA_MAX_ATOMS atoms and PME
// grids of at most NA_MAX_N points per side; every GPU that loads this library holds it
// (about 7.5 MB) until the process exits.

namespace {

constexpr int NA_MAX_ATOMS = 65536;
constexpr int NA_MAX_N = 64;
constexpr int NA_MAX_COLS = (NA_MAX_N / 2 + 1) * ((NA_MAX_N + NB_TKF - 1) / NB_TKF);
constexpr int NA_MAX_TAB = 3 * 8 * NA_MAX_N;
constexpr size_t na_up(size_t x) { return (x + 255) & ~(size_t)255; }

// arena regions (byte offsets, 256-byte aligned)
constexpr size_t NA_POS = 0;
constexpr size_t NA_Q = NA_POS + na_up(sizeof(float4) * NA_MAX_ATOMS);
constexpr size_t NA_REP = NA_Q + na_up(sizeof(float) * NA_MAX_ATOMS);
constexpr size_t NA_FR = NA_REP + na_up(sizeof(int) * NA_MAX_ATOMS);
constexpr size_t NA_ZSLOT = NA_FR + na_up(sizeof(float4) * NA_MAX_ATOMS);
constexpr size_t NA_ZATOMS = NA_ZSLOT + na_up(sizeof(int) * NA_MAX_ATOMS);
constexpr size_t NA_PART = NA_ZATOMS + na_up(sizeof(int) * NA_MAX_ATOMS);
constexpr size_t NA_ZCOUNT = NA_PART + na_up(sizeof(float) * 12 * NA_MAX_ATOMS);
constexpr size_t NA_ZSTART = NA_ZCOUNT + na_up(sizeof(int) * (NA_MAX_N + 1));
constexpr size_t NA_GRID = NA_ZSTART + na_up(sizeof(int) * (NA_MAX_N + 1));
constexpr size_t NA_ECOL = NA_GRID + na_up(sizeof(float2) * ((NA_MAX_N / 2 + 1) * NA_MAX_N * NA_MAX_N + 2));
constexpr size_t NA_PLANES = NA_ECOL + na_up(sizeof(double) * NA_MAX_COLS);
constexpr size_t NA_COLS = NA_PLANES + na_up(sizeof(PlaneWork) * NA_MAX_N);
constexpr size_t NA_COLBEG = NA_COLS + na_up(sizeof(ColWork) * NA_MAX_COLS);
constexpr size_t NA_PLANS = NA_COLBEG + na_up(sizeof(int) * 2);
constexpr size_t NA_REPPLAN = NA_PLANS + na_up(sizeof(FftPlanDev) * 3);
constexpr size_t NA_TW = NA_REPPLAN + na_up(sizeof(int) * 3);
constexpr size_t NA_TAB = NA_TW + na_up(sizeof(float2) * 3 * NA_MAX_N);
constexpr size_t NA_BSP = NA_TAB + na_up(sizeof(int2) * NA_MAX_TAB);
constexpr size_t NA_ETAB = NA_BSP + na_up(sizeof(float) * 3 * NA_MAX_N);
constexpr size_t NA_REPS = NA_ETAB + na_up(sizeof(float) * 3 * NA_MAX_N);
constexpr size_t NA_EOUT = NA_REPS + na_up(sizeof(RepDev));
constexpr size_t NA_STATUS = NA_EOUT + na_up(sizeof(double));
constexpr size_t NA_BYTES = NA_STATUS + na_up(sizeof(int) * 8);

static __device__ __align__(256) unsigned char g_pme_scratch[NA_BYTES];

std::mutex g_na_mu;
constexpr int NA_MAX_DEVICES = 64;
unsigned char *g_na_base[NA_MAX_DEVICES] = {};

__global__ void k_na_load(int natom, const double *__restrict__ coor, const double *__restrict__ q,
                          float4 *__restrict__ pos, float *__restrict__ sq, int *__restrict__ srep)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natom) return;
    pos[a] = make_float4((float)coor[3 * (size_t)a], (float)coor[3 * (size_t)a + 1], (float)coor[3 * (size_t)a + 2], 0.f);
    sq[a] = (float)q[a];
    srep[a] = 0;
}

// int32 plane scale from the largest charge (same rule as the handle path)
__global__ void k_na_scale(int natom, const double *__restrict__ q, RepDev *__restrict__ reps)
{
    __shared__ double sh[256];
    double m = 0;
    for (int a = threadIdx.x; a < natom; a += blockDim.x) m = fmax(m, fabs(q[a]));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int k = nb_spread_exp(sh[0] * reps[0].fcd);
        reps[0].spread_scale = (float)ldexp(1.0, k);
        reps[0].spread_inv = (float)ldexp(1.0, -k);
        const double s216 = ldexp(1.0, k) / 216.0;
        reps[0].spread216 = (float)s216;
        const double c = s216 / (double)reps[0].spread216;
        reps[0].pme_qcorr = c * c;
    }
}

// gradient from the four per-plane slots (grad_sum, pot/ewald_receip.f:815-970); overwrites dpot
__global__ void k_na_grad(int natom, const RepDev *__restrict__ reps, const double *__restrict__ q,
                          const float *__restrict__ part, double *__restrict__ dpot)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natom) return;
    const RepDev &R = reps[0];
    const float4 p = ((const float4 *)part)[a];   // k_pme_gather_f: one (x, y, z) per atom
    const double pg[3] = {(double)p.x, (double)p.y, (double)p.z};
    double qf = q[a] * R.fcd;
    dpot[3 * (size_t)a] = qf * R.n1 * R.invLd[0] * pg[0];
    dpot[3 * (size_t)a + 1] = qf * R.n2 * R.invLd[1] * pg[1];
    dpot[3 * (size_t)a + 2] = qf * R.n3 * R.invLd[2] * pg[2];
}

__global__ void k_na_energy(int ncol, const double *__restrict__ e_col, double *__restrict__ out)
{
    __shared__ double sh[256];
    double v = 0;
    for (int w = threadIdx.x; w < ncol; w += blockDim.x) v += e_col[w];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = 0.5 * sh[0];
}

}  // namespace

extern "C" int moil_nb_pme_noalloc(const double *d_coor, const double *d_q, int natom, const double *box,
                                   const int *grid, double alpha, double eps, double *d_dpot, double *e_recip,
                                   void *stream_v)
{
    if (!d_coor || !d_q || !box || !grid || !d_dpot || !e_recip) return MOIL_NB_ERR_ARG;
    if (natom < 1 || natom > NA_MAX_ATOMS || !(alpha > 0) || !(eps > 0)) return MOIL_NB_ERR_ARG;
    for (int d = 0; d < 3; ++d) {
        FftPlanDev p;
        if (!(box[d] > 0) || grid[d] < 4 || grid[d] > NA_MAX_N || !make_plan(grid[d], &p, nullptr, false) ||
            !make_plan(grid[d], &p, nullptr, true))
            return MOIL_NB_ERR_GRID;
    }
    cudaStream_t stream = (cudaStream_t)stream_v;
    // an error the caller's own earlier work left pending is reported and left in place
    if (cudaPeekAtLastError() != cudaSuccess) return MOIL_NB_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return MOIL_NB_ERR_CUDA;
    unsigned char *base = nullptr;
    {
        // first call on this device: resolve the device address of the scratch array (the
        // symbol itself is only a host-side stand-in and must not be handed to a kernel)
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_base[dev]) {
            void *ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_pme_scratch) != cudaSuccess || !ptr) return MOIL_NB_ERR_CUDA;
            g_na_base[dev] = (unsigned char *)ptr;
        }
        base = g_na_base[dev];
    }
    const int n1 = grid[0], n2 = grid[1], n3 = grid[2];
    {
        // the planes of this grid must fit the device's shared memory per block
        int optin = 0;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            return MOIL_NB_ERR_CUDA;
        if (plane_fwd_smem<float>(n1, n2) > (size_t)optin || plane_inv_smem<float>(n1, n2) > (size_t)optin ||
            zconv_smem<float>(n3) > (size_t)optin)
            return MOIL_NB_ERR_GRID;
    }
    // shared-memory limits for this grid (raise only; other handles may need more)
    if (raise_pme_limits<float>(plane_fwd_smem<float>(n1, n2), zconv_smem<float>(n3),
                                plane_inv_smem<float>(n1, n2)) != cudaSuccess)
        return MOIL_NB_ERR_CUDA;
    // one-replica constants, FFT plans and tables, B-spline moduli, work lists (host side)
    RepDev R;
    memset(&R, 0, sizeof(R));
    for (int d = 0; d < 3; ++d) {
        R.Ld[d] = box[d];
        R.L[d] = (float)box[d];
        R.invLd[d] = 1.0 / box[d];
        R.invL[d] = (float)(1.0 / box[d]);
        R.Llo[d] = (float)(box[d] - (double)R.L[d]);
    }
    R.n1 = n1; R.n2 = n2; R.n3 = n3; R.n1h = n1 / 2 + 1;
    R.epstmp = NB_KOFDIE / eps;
    R.fcd = sqrt(R.epstmp);
    R.fc = (float)R.fcd;
    R.alpha = (float)alpha;
    R.alphad = alpha;
    R.pme_fac = M_PI * M_PI / (alpha * alpha);
    R.pivol = M_PI * box[0] * box[1] * box[2];
    nb_pme_fp32_consts(&R);
    R.pme_qcorr = 1.0;    // the charges stay on the device: no rounding correction
    R.natom = natom;
    FftPlanDev plans[3];
    int rep_plan[3];
    float2 tw[3 * NA_MAX_N];
    std::vector<int2> tab;
    float bsp[3 * NA_MAX_N];
    int ntw = 0;
    for (int d = 0; d < 3; ++d) {
        int tab0 = (int)tab.size();
        make_plan(grid[d], &plans[d], &tab, d == 2);     // the z columns take the wide radix set
        plans[d].tab0 = tab0;
        plans[d].tw0 = ntw;
        for (int t = 0; t < grid[d]; ++t) {
            double ang = -2.0 * M_PI * (double)t / (double)grid[d];
            tw[ntw++] = make_float2((float)cos(ang), (float)sin(ang));
        }
        rep_plan[d] = d;
    }
    if ((int)tab.size() > NA_MAX_TAB) return MOIL_NB_ERR_GRID;
    double bspd[3 * NA_MAX_N];
    nb_bsp_moduli(n1, bspd);
    nb_bsp_moduli(n2, bspd + n1);
    nb_bsp_moduli(n3, bspd + n1 + n2);
    for (int k = 0; k < n1 + n2 + n3; ++k) bsp[k] = (float)bspd[k];
    float etab[3 * NA_MAX_N];
    nb_pme_etab(R, bspd, etab);
    NbCtx tmp;
    tmp.stream = stream;
    tmp.nrep = 1;
    tmp.nsite = natom;
    tmp.nzbin = n3;
    for (int z = 0; z < n3; ++z) tmp.planes.push_back(PlaneWork{0, z});
    for (int kx = 0; kx < R.n1h; ++kx)
        push_col_runs(tmp.cols, 0, kx, n2, NB_TKF);
    int col_begin[2] = {0, (int)tmp.cols.size()};
    tmp.smem_plane_fwd = plane_fwd_smem<float>(n1, n2);
    tmp.smem_plane_inv = plane_inv_smem<float>(n1, n2);
    tmp.smem_zconv = zconv_smem<float>(n3);
    tmp.d_pos = base + NA_POS;
    tmp.d_site_q = base + NA_Q;
    tmp.d_site_rep = (int *)(base + NA_REP);
    tmp.d_fr = base + NA_FR;
    tmp.d_zslot = (int *)(base + NA_ZSLOT);
    tmp.d_zatoms = (int *)(base + NA_ZATOMS);
    tmp.d_part = base + NA_PART;
    tmp.d_zcount = (int *)(base + NA_ZCOUNT);
    tmp.d_zstart = (int *)(base + NA_ZSTART);
    tmp.d_grid = base + NA_GRID;
    tmp.d_e_col = (double *)(base + NA_ECOL);
    tmp.d_planes = (PlaneWork *)(base + NA_PLANES);
    tmp.d_cols = (ColWork *)(base + NA_COLS);
    tmp.d_col_begin = (int *)(base + NA_COLBEG);
    tmp.d_plans = (FftPlanDev *)(base + NA_PLANS);
    tmp.d_rep_plan = (int *)(base + NA_REPPLAN);
    tmp.d_tw = base + NA_TW;
    tmp.d_tab = (int2 *)(base + NA_TAB);
    tmp.d_bsp = base + NA_BSP;
    tmp.d_etab = (float *)(base + NA_ETAB);
    tmp.d_reps = (RepDev *)(base + NA_REPS);
    tmp.d_status = (int *)(base + NA_STATUS);
    double *d_eout = (double *)(base + NA_EOUT);
#define NA_CP(dst, src, bytes)                                                                       \
    if (cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyHostToDevice, stream) != cudaSuccess)      \
        return MOIL_NB_ERR_CUDA;
    NA_CP(tmp.d_reps, &R, sizeof(R));
    NA_CP(tmp.d_plans, plans, sizeof(plans));
    NA_CP(tmp.d_rep_plan, rep_plan, sizeof(rep_plan));
    NA_CP(tmp.d_tw, tw, sizeof(float2) * ntw);
    NA_CP(tmp.d_tab, tab.data(), sizeof(int2) * tab.size());
    NA_CP(tmp.d_bsp, bsp, sizeof(float) * (n1 + n2 + n3));
    NA_CP(tmp.d_etab, etab, sizeof(float) * (n1 + n2 + n3));
    NA_CP(tmp.d_planes, tmp.planes.data(), sizeof(PlaneWork) * tmp.planes.size());
    NA_CP(tmp.d_cols, tmp.cols.data(), sizeof(ColWork) * tmp.cols.size());
    NA_CP(tmp.d_col_begin, col_begin, sizeof(col_begin));
#undef NA_CP
    k_na_load<<<(natom + 255) / 256, 256, 0, stream>>>(natom, d_coor, d_q, (float4 *)tmp.d_pos,
                                                       (float *)tmp.d_site_q, tmp.d_site_rep);
    k_na_scale<<<1, 256, 0, stream>>>(natom, d_q, tmp.d_reps);
    pme_t<float>(&tmp);
    k_na_grad<<<(natom + 255) / 256, 256, 0, stream>>>(natom, tmp.d_reps, d_q, (const float *)tmp.d_part, d_dpot);
    k_na_energy<<<1, 256, 0, stream>>>((int)tmp.cols.size(), tmp.d_e_col, d_eout);
    // a launch that failed is reported before waiting for the stream (the error stays pending
    // for the caller to read)
    if (cudaPeekAtLastError() != cudaSuccess) return MOIL_NB_ERR_CUDA;
    if (cudaMemcpyAsync(e_recip, d_eout, sizeof(double), cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        return MOIL_NB_ERR_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess || cudaPeekAtLastError() != cudaSuccess) return MOIL_NB_ERR_CUDA;
    return MOIL_NB_OK;
}
