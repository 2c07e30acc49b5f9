// nb_fft.cuh -- complex helpers and the in-register DFT codelets of the PME transforms.
//
// Every codelet computes the forward DFT X[k] = sum_n x[n] exp(-2 pi i n k / R) of R values
// in place.  Radices 2, 3, 4, 5 are direct butterflies; 6 and 10 are prime-factor (Good-Thomas)
// compositions of 2 x 3 and 2 x 5, which need no twiddle factors: input n = (N2 n1 + N1 n2)
// mod R, output k = the CRT index of (k1 mod N1, k2 mod N2); 8 and 9 are Cooley-Tukey
// compositions (2 x 4 and 3 x 3, decimation in time) with their few twiddles as constants.
// They let a line of up to 100 points be transformed in two Stockham passes.
#pragma once

template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b)
{
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
// multiply by -i
template <typename C> __host__ __device__ __forceinline__ C cmi(C a) { C r; r.x = a.y; r.y = -a.x; return r; }
// multiply by the constant (c - i s) = exp(-i phi) for c = cos phi, s = sin phi
template <typename C, typename T> __host__ __device__ __forceinline__ C crot(C a, T c, T s)
{
    C r;
    r.x = a.x * c + a.y * s;
    r.y = a.y * c - a.x * s;
    return r;
}

// forward DFT butterflies, W_R = exp(-2 pi i / R)
template <typename C> __host__ __device__ __forceinline__ void bfly2(C *v)
{
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
template <typename C> __host__ __device__ __forceinline__ void bfly4(C *v)
{
    C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]), t2 = cadd(v[1], v[3]), t3 = cmi(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
}
template <typename C> __host__ __device__ __forceinline__ void bfly3(C *v)
{
    typedef decltype(v[0].x) T;
    const T h = (T)0.86602540378443864676;   // sqrt(3)/2
    C s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    C m;
    m.x = v[0].x - (T)0.5 * s.x;
    m.y = v[0].y - (T)0.5 * s.y;
    C r0 = cadd(v[0], s);
    C r1, r2;
    r1.x = m.x + h * d.y; r1.y = m.y - h * d.x;
    r2.x = m.x - h * d.y; r2.y = m.y + h * d.x;
    v[0] = r0; v[1] = r1; v[2] = r2;
}
template <typename C> __host__ __device__ __forceinline__ void bfly5(C *v)
{
    typedef decltype(v[0].x) T;
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;   // cos(2pi/5), cos(4pi/5)
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;    // sin(2pi/5), sin(4pi/5)
    C a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]), a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    C x0 = v[0];
    C p1, p2;
    p1.x = x0.x + c1 * a1.x + c2 * a2.x; p1.y = x0.y + c1 * a1.y + c2 * a2.y;
    p2.x = x0.x + c2 * a1.x + c1 * a2.x; p2.y = x0.y + c2 * a1.y + c1 * a2.y;
    C q1, q2;   // the sine combinations; results are p -/+ i q
    q1.x = s1 * b1.x + s2 * b2.x; q1.y = s1 * b1.y + s2 * b2.y;
    q2.x = s2 * b1.x - s1 * b2.x; q2.y = s2 * b1.y - s1 * b2.y;
    v[0].x = x0.x + a1.x + a2.x; v[0].y = x0.y + a1.y + a2.y;
    C mq1 = cmi(q1), mq2 = cmi(q2);
    v[1] = cadd(p1, mq1);
    v[4] = csub(p1, mq1);
    v[2] = cadd(p2, mq2);
    v[3] = csub(p2, mq2);
}
// 6 = 2 x 3, prime factor: a = x(0, 2, 4), b = x(3, 5, 1); X(0, 4, 2) = A + B, X(3, 1, 5) = A - B
template <typename C> __host__ __device__ __forceinline__ void bfly6(C *v)
{
    C a[3] = {v[0], v[2], v[4]}, b[3] = {v[3], v[5], v[1]};
    bfly3(a);
    bfly3(b);
    v[0] = cadd(a[0], b[0]); v[3] = csub(a[0], b[0]);
    v[4] = cadd(a[1], b[1]); v[1] = csub(a[1], b[1]);
    v[2] = cadd(a[2], b[2]); v[5] = csub(a[2], b[2]);
}
// 10 = 2 x 5, prime factor: a = x(0, 2, 4, 6, 8), b = x(5, 7, 9, 1, 3);
// X(0, 6, 2, 8, 4) = A + B, X(5, 1, 7, 3, 9) = A - B
template <typename C> __host__ __device__ __forceinline__ void bfly10(C *v)
{
    C a[5] = {v[0], v[2], v[4], v[6], v[8]}, b[5] = {v[5], v[7], v[9], v[1], v[3]};
    bfly5(a);
    bfly5(b);
    v[0] = cadd(a[0], b[0]); v[5] = csub(a[0], b[0]);
    v[6] = cadd(a[1], b[1]); v[1] = csub(a[1], b[1]);
    v[2] = cadd(a[2], b[2]); v[7] = csub(a[2], b[2]);
    v[8] = cadd(a[3], b[3]); v[3] = csub(a[3], b[3]);
    v[4] = cadd(a[4], b[4]); v[9] = csub(a[4], b[4]);
}
// 8 = 2 x 4, decimation in time: E, O = DFT4 of the even and odd samples, O(k) *= W_8^k,
// X(k) = E(k) + O(k), X(k + 4) = E(k) - O(k)
template <typename C> __host__ __device__ __forceinline__ void bfly8(C *v)
{
    typedef decltype(v[0].x) T;
    const T r = (T)0.70710678118654752440;   // sqrt(1/2)
    C e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    bfly4(e);
    bfly4(o);
    o[1] = crot(o[1], r, r);
    o[2] = cmi(o[2]);
    o[3] = crot(o[3], -r, r);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = cadd(e[k], o[k]);
        v[k + 4] = csub(e[k], o[k]);
    }
}
// 9 = 3 x 3, decimation in time: Y_m = DFT3 of x(m, m + 3, m + 6), Y_m(k) *= W_9^(m k),
// X(k + 3 j) = DFT3 over m of Y_m(k) at j
template <typename C> __host__ __device__ __forceinline__ void bfly9(C *v)
{
    typedef decltype(v[0].x) T;
    const T c1 = (T)0.76604444311897803520, s1 = (T)0.64278760968653932632;    // 2pi/9
    const T c2 = (T)0.17364817766693034885, s2 = (T)0.98480775301220805936;    // 4pi/9
    const T c4 = (T)-0.93969262078590838405, s4 = (T)0.34202014332566873304;   // 8pi/9
    C y0[3] = {v[0], v[3], v[6]}, y1[3] = {v[1], v[4], v[7]}, y2[3] = {v[2], v[5], v[8]};
    bfly3(y0);
    bfly3(y1);
    bfly3(y2);
    y1[1] = crot(y1[1], c1, s1);
    y1[2] = crot(y1[2], c2, s2);
    y2[1] = crot(y2[1], c2, s2);
    y2[2] = crot(y2[2], c4, s4);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        C z[3] = {y0[k], y1[k], y2[k]};
        bfly3(z);
        v[k] = z[0];
        v[k + 3] = z[1];
        v[k + 6] = z[2];
    }
}

template <int R, typename C> __host__ __device__ __forceinline__ void bfly(C *v)
{
    if (R == 2) bfly2(v);
    else if (R == 3) bfly3(v);
    else if (R == 4) bfly4(v);
    else if (R == 5) bfly5(v);
    else if (R == 6) bfly6(v);
    else if (R == 8) bfly8(v);
    else if (R == 9) bfly9(v);
    else bfly10(v);
}
