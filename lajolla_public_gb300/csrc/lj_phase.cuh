// Phase functions on the device (FP32): src/phase_functions/isotropic.inl:1-15
// and src/phase_functions/henyeygreenstein.inl:1-48 (eval == pdf; inverse-CDF
// sampling in Frame(dir_in), uniform sphere when |g| < 1e-3).
#pragma once

#include "lj_common.cuh"

namespace lj {

LJ_HD float hg_eval(float g, V3 wi, V3 wo) {
    float den = 1.0f + g * g + 2.0f * g * dot(wi, wo);
    return kInvFourPi * (1.0f - g * g) / (den * sqrtf(den));
}
LJ_HD V3 uniform_sphere(float u0, float u1) {
    float z = 1.0f - 2.0f * u0;
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float sp, cp;
    sincosf(kTwoPi * u1, &sp, &cp);
    return V3{r * cp, r * sp, z};
}
LJ_HD V3 hg_sample(float g, V3 wi, float u0, float u1) {
    if (fabsf(g) < 1e-3f) return uniform_sphere(u0, u1);
    float tmp = (g * g - 1.0f) / (2.0f * u0 * g - (g + 1.0f));
    float ce = (tmp * tmp - (1.0f + g * g)) / (2.0f * g);
    float se = sqrtf(fmaxf(1.0f - ce * ce, 0.0f));
    float sp, cp;
    sincosf(kTwoPi * u1, &sp, &cp);
    Frame f = frame_from_n(wi);
    return to_world(f, V3{se * cp, se * sp, ce});
}
// kind: 0 isotropic, 1 Henyey-Greenstein
LJ_HD float phase_eval(int kind, float g, V3 wi, V3 wo) {
    return kind == 1 ? hg_eval(g, wi, wo) : kInvFourPi;
}
LJ_HD V3 phase_sample(int kind, float g, V3 wi, float u0, float u1) {
    return kind == 1 ? hg_sample(g, wi, u0, u1) : uniform_sphere(u0, u1);
}

}  // namespace lj
