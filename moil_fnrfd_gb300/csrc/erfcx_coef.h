/* generated by fit_erfcx.py: erfcx(x) ~= t * sum_k C[k] u^k, t = 1/(1 + P x), u = A t + B */
/* FP32 relative error on [0, 4.5]: max 3.49e-07, rms 8.63e-08 */
#pragma once
#define ERFCX_P 5.500000000e-01f
#define ERFCX_A 2.808080808e+00f
#define ERFCX_B -1.808080808e+00f
#define ERFCX_NC 8
#define ERFCX_COEFS {6.617053130e-01f, 2.925414369e-01f, 5.375989220e-02f, -5.832119097e-03f, -2.772902939e-03f, 5.236826469e-04f, 1.250510914e-04f, -5.035757194e-05f}
