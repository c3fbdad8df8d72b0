/* Exhaustive check of the float forms kittlespt_gb300/csrc/kpt_fsr.cu uses in
 * place of the reference's double-precision FSR expressions (upscale.cuh):
 * for every float input in the range the kernel can see, the float form
 * must give the same float as the double form.  Prints the number of
 * mismatches per expression; all must be 0.  Compiled without contraction
 * (-ffp-contract=off); fmaf is the correctly rounded fused multiply-add, as
 * on the GPU. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

#define NT 16
static const float CL4 = -0x1.99999ap-28f;   /* (float)(0.4 - (double)0.4f) */
static long long bad[NT][4];

/* the tap weight's first factor: (float)(0.4 * (double)d2 - 1.0), then
 * squared and 1.5625 * wB - 0.5625 (double in the reference, one fma here) */
static float wb_ref(float d2) {
    float w = (float)(0.4 * (double)d2 - 1.0);
    w *= w;
    return (float)(1.5625 * (double)w - 0.5625);
}
static float wb_float(float d2) {
    const float ph = 0.4f * d2, pl = fmaf(0.4f, d2, -ph), tt = fmaf(CL4, d2, pl);
    const float sm = ph + -1.0f, bb = sm - ph, er = (ph - (sm - bb)) + (-1.0f - bb);
    float w = sm + (er + tt);
    w *= w;
    return fmaf(1.5625f, w, -0.5625f);
}

static void* work(void* arg) {
    const int t = (int)(intptr_t)arg;
    /* d2 = min(|v|^2, clp) with clp = 1 / lob <= 1 / 0.21 */
    for (uint32_t u = (uint32_t)t; u <= u_of(4.8f); u += NT)
        if (u_of(wb_float(f_of(u))) != u_of(wb_ref(f_of(u)))) bad[t][0]++;
    /* len in [0, 1]: 1. - .5 * len */
    for (uint32_t u = (uint32_t)t; u <= u_of(1.0f); u += NT) {
        const float len = f_of(u);
        if (u_of((float)(1.0 - 0.5 * (double)len)) != u_of(1.0f - 0.5f * len)) bad[t][1]++;
    }
    /* lob = (float)(.5 - .29 * len) in [0.21, 0.5]: 1. / lob */
    for (uint32_t u = u_of(0.2f) + (uint32_t)t; u <= u_of(0.51f); u += NT) {
        const float lob = f_of(u);
        if (u_of((float)(1.0 / (double)lob)) != u_of(1.0f / lob)) bad[t][2]++;
    }
    return 0;
}

int main(void) {
    pthread_t th[NT];
    long long b[4] = {0, 0, 0, 0};
    for (int t = 0; t < NT; ++t) pthread_create(&th[t], 0, work, (void*)(intptr_t)t);
    for (int t = 0; t < NT; ++t) {
        pthread_join(th[t], 0);
        for (int k = 0; k < 3; ++k) b[k] += bad[t][k];
    }
    printf("tap_weight %lld one_minus_half_len %lld inv_lob %lld\n", b[0], b[1], b[2]);
    return 0;
}
