/*
 * nglod_oracle.c -- C restatements used as the bit-exact oracle (TEST
 * INFRASTRUCTURE ONLY; loaded by oracle/cref.py from tests and the CPU
 * baseline, never by the nglod_gb300 package).
 *
 * Compiled with -ffp-contract=off so that every float operation rounds as
 * written; fused multiply-adds appear only where the reference source calls
 * fmaf explicitly or where a contraction is stated in the comment.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

/* Ray vs [-1,1]^3, sdf-net/lib/extensions/sol_nglod/sol_nglod_kernel.cu:92-150:
 * invdir = (float)(1.0 / (double)d); sgn = signbit(d) ? 1 : -1; rays with
 * max|o| < 1 are skipped; d_k = (sgn_k - o_k) * invdir_k; face k passes when
 * d_k >= 0 and both other coordinates of fmaf(dir, d_k, o) are inside (-1, 1);
 * the first passing face in x, y, z order is taken if its d < 500, and then
 * x = fmaf(dir, d, o), t = d, hit = 1.  Otherwise x = o, t = 0, hit = 0. */
void oracle_aabb(const float *ro, const float *rd, int64_t n, float *x, float *t, uint8_t *hit) {
    for (int64_t i = 0; i < n; ++i) {
        const float o[3] = {ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]};
        const float d[3] = {rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]};
        float inv[3], sg[3], dd[3];
        int k;
        for (k = 0; k < 3; ++k) {
            inv[k] = (float)(1.0 / (double)d[k]);
            sg[k] = signbit(d[k]) ? 1.0f : -1.0f;
        }
        x[3 * i] = o[0];
        x[3 * i + 1] = o[1];
        x[3 * i + 2] = o[2];
        t[i] = 0.0f;
        hit[i] = 0;
        const float cmax = fmaxf(fmaxf(fabsf(o[0]), fabsf(o[1])), fabsf(o[2]));
        if (cmax < 1.0f) continue;
        for (k = 0; k < 3; ++k) {
            const float a = sg[k] - o[k];
            dd[k] = a * inv[k];
        }
        static const int other[3][2] = {{1, 2}, {0, 2}, {0, 1}};
        int face = -1;
        for (k = 0; k < 3 && face < 0; ++k) {
            const int b = other[k][0], c = other[k][1];
            const float lb = fmaf(d[b], dd[k], o[b]);
            const float lc = fmaf(d[c], dd[k], o[c]);
            if (dd[k] >= 0.0f && fabsf(lb) < 1.0f && fabsf(lc) < 1.0f) face = k;
        }
        if (face < 0) continue;
        const float dist = dd[face];
        if (!(dist < 500.0f)) continue;
        hit[i] = 1;
        t[i] = dist;
        for (k = 0; k < 3; ++k) x[3 * i + k] = fmaf(d[k], dist, o[k]);
    }
}
