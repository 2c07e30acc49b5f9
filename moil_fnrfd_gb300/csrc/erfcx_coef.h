/* generated by fit_erfcx.py: erfcx(x) ~= t * sum_k C[k] u^k, t = 1/(1 + P x), u = A t + B */
/* FP32 relative error on [0, 4.5]: max 3.73e-07, rms 9.00e-08 */
#pragma once
#define ERFCX_P 4.704700000e-01f
#define ERFCX_A 2.944681796e+00f
#define ERFCX_B -1.944681796e+00f
#define ERFCX_NC 9
#define ERFCX_COEFS {6.109123249e-01f, 3.034594872e-01f, 8.253738631e-02f, 5.967158690e-03f, -2.695183977e-03f, -3.349032720e-04f, 1.546260985e-04f, 8.643689531e-06f, -9.546006234e-06f}
