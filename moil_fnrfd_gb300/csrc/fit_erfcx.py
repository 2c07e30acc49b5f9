"""Generate the FP32 coefficients of erfcx(x) = erfc(x) * exp(x^2) used by the
real-space kernels (written to ``erfcx_coef.h``).

Method: the substitution t = 1 / (1 + p x) of Hastings (1955), used in
Abramowitz & Stegun 7.1.26 (there with p = 0.47047; p = 0.55 here, the value
that minimises the degree-7 error); erfcx(x) is written as
t * P(u), u = a t + b the affine map of t in [1/(1 + p X), 1] onto [-1, 1],
and P of degree 7 is a least-squares fit of the *relative* error in a
Chebyshev basis of u at 8000 Chebyshev nodes in x on [0, X], X = 4.5
(alpha * r_cut is 3.15 for alpha 0.35 / 9 Å and 3.2 for 0.32 / 10 Å).  The
Chebyshev series is converted to monomials in u for Horner evaluation.

Reference values come from scipy.special.erfcx (double precision).  Measured
FP32 error of the Horner evaluation over [0, 4.5]: max 3.5e-7, rms 8.6e-8
relative (degree 8 with p = 0.47047: 3.7e-7, 9.0e-8; degree 6: 6.5e-7 at best).  Run:  python fit_erfcx.py > erfcx_coef.h
"""
import numpy as np
from scipy.special import erfcx

X_MAX = 4.5
P_SUB = 0.55
DEG = 7


def fit():
    n = 8000
    xs = X_MAX / 2 * (1 - np.cos(np.pi * (np.arange(n) + 0.5) / n))
    t = 1 / (1 + P_SUB * xs)
    r = erfcx(xs)
    tl, th = 1 / (1 + P_SUB * X_MAX), 1.0
    a = 2 / (th - tl)
    b = -(tl + th) / (th - tl)
    v = np.polynomial.chebyshev.chebvander(a * t + b, DEG) * t[:, None]
    cc, *_ = np.linalg.lstsq(v / r[:, None], np.ones_like(r), rcond=None)
    cu = np.polynomial.chebyshev.cheb2poly(cc)
    return a, b, cu


def fp32_error(a, b, cu):
    cu32 = cu.astype(np.float32)
    xt = np.linspace(0, X_MAX, 400001)
    tt = (np.float32(1) / (np.float32(1) + np.float32(P_SUB) * xt.astype(np.float32))).astype(np.float32)
    uu = (np.float32(a) * tt + np.float32(b)).astype(np.float32)
    pp = np.full_like(tt, cu32[-1])
    for k in range(len(cu32) - 2, -1, -1):
        pp = (pp * uu + cu32[k]).astype(np.float32)
    rel = (pp * tt).astype(np.float64) / erfcx(xt) - 1
    return np.abs(rel).max(), np.sqrt(np.mean(rel ** 2))


def main():
    a, b, cu = fit()
    mx, rms = fp32_error(a, b, cu)
    print("/* generated by fit_erfcx.py: erfcx(x) ~= t * sum_k C[k] u^k, t = 1/(1 + P x), u = A t + B */")
    print(f"/* FP32 relative error on [0, {X_MAX}]: max {mx:.2e}, rms {rms:.2e} */")
    print("#pragma once")
    print(f"#define ERFCX_P {P_SUB:.9e}f")
    print(f"#define ERFCX_A {a:.9e}f")
    print(f"#define ERFCX_B {b:.9e}f")
    print(f"#define ERFCX_NC {len(cu)}")
    print("#define ERFCX_COEFS {" + ", ".join(f"{c:.9e}f" for c in cu) + "}")


if __name__ == "__main__":
    main()
