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

/* ------------------------------------------------------------------------ */
/* SPC ray/octree traversal: include/spc/spc/spc_raytrace_cuda_kernel.cu    */
/* ------------------------------------------------------------------------ */
#include <stdlib.h>

/* Front-to-back order of the children of a voxel for a ray whose origin is in
 * octant `code`: sorted by Hamming distance of the child index to code, ties
 * by index (the Order table, spc_raytrace_cuda_kernel.cu:39-47). */
static int child_order(int code, int rank) {
    int seen = 0;
    for (int dist = 0; dist <= 3; ++dist)
        for (int j = 0; j < 8; ++j)
            if (__builtin_popcount((unsigned)(j ^ code)) == dist) {
                if (seen == rank) return j;
                ++seen;
            }
    return 0;
}

void oracle_child_order_table(uint8_t *out64) {
    for (int c = 0; c < 8; ++c)
        for (int r = 0; r < 8; ++r) out64[8 * c + r] = (uint8_t)child_order(c, r);
}

/* d_FaceEval (85-105) as nvcc contracts a*i + b*j + c in the reference build:
 * fma(b, j, a*i) + c; then +a, +b, +b.  The contraction was pinned on the GPU
 * against the reference kernel's own decisions (135M ray/voxel candidates of a
 * 1920x1080 frame, octree levels 0-7): of the nine legal forms of crs3 and of
 * this sum, only fma(u, v, -(w*z)) with fma(b, j, a*i) + c agrees with all. */
static int face_straddles(float fi, float fj, float a, float b, float c) {
    const float r0 = fmaf(b, fj, a * fi) + c;
    const float r1 = r0 + a;
    const float r2 = r0 + b;
    const float r3 = r1 + b;
    const float r[4] = {r0, r1, r2, r3};
    float mn = 1.0f, mx = -1.0f;
    for (int k = 0; k < 4; ++k) {
        if (r[k] < mn) mn = r[k];
        if (r[k] > mx) mx = r[k];
    }
    return mn <= 0.0f && mx >= 0.0f;
}

/* d_Decide (108-138): ray mapped to [0,1]^3, o' x d' with fma(u, v, -(w*z)). */
static int ray_hits_voxel(const float *org, const float *dir, int64_t r, const int16_t *p, int level) {
    const float ox = fmaf(0.5f, org[3 * r], 0.5f), oy = fmaf(0.5f, org[3 * r + 1], 0.5f),
                oz = fmaf(0.5f, org[3 * r + 2], 0.5f);
    const float dx = 0.5f * dir[3 * r], dy = 0.5f * dir[3 * r + 1], dz = 0.5f * dir[3 * r + 2];
    const float cx = fmaf(oy, dz, -(dy * oz));
    const float cy = fmaf(oz, dx, -(dz * ox));
    const float cz = fmaf(ox, dy, -(dx * oy));
    const float s1 = ldexpf(1.0f, -level);
    const float s2 = s1 * s1;
    const float px = (float)(uint16_t)p[0], py = (float)(uint16_t)p[1], pz = (float)(uint16_t)p[2];
    return face_straddles(py, pz, -s2 * dz, s2 * dy, s1 * cx) && face_straddles(px, pz, s2 * dz, -s2 * dx, s1 * cy) &&
           face_straddles(px, py, -s2 * dy, s2 * dx, s1 * cz);
}

/* d_Subdivide's origin octant (157-167), formed in double as the reference does. */
static int origin_octant(const float *org, int64_t r, const int16_t *p, int level) {
    const double sc = ldexp(1.0, -level);
    int code = 0;
    if ((float)((double)fmaf(0.5f, org[3 * r], 0.5f) - sc * ((double)p[0] + 0.5)) > 0.0f) code = 4;
    if ((float)((double)fmaf(0.5f, org[3 * r + 1], 0.5f) - sc * ((double)p[1] + 0.5)) > 0.0f) code += 2;
    if ((float)((double)fmaf(0.5f, org[3 * r + 2], 0.5f) - sc * ((double)p[2] + 0.5)) > 0.0f) code += 1;
    return code;
}

/* spc_raytrace (spc_raytrace_cuda_kernel.cu:194-265): returns the number of
 * nuggets at target_level written to out[cap][2] (ray, level-local voxel),
 * or -1 if more than cap would be needed at some level. */
int64_t oracle_spc_raytrace(const uint8_t *octree, const int16_t *points, const uint32_t *prefix,
                            const int32_t *pyramid, int level, int target, const float *org, const float *dir,
                            int64_t n, int32_t *out, int64_t cap) {
    const int32_t *psum = pyramid + level + 2;
    int32_t *cur = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)(n > 0 ? n : 1));
    int64_t num = n;
    for (int64_t i = 0; i < n; ++i) {
        cur[2 * i] = (int32_t)i;
        cur[2 * i + 1] = 0;
    }
    for (int l = 0; l <= target; ++l) {
        const int64_t off0 = psum[l], off1 = psum[l + 1];
        int64_t total = 0;
        for (int64_t i = 0; i < num; ++i) {
            const int16_t *p = points + 4 * (off0 + cur[2 * i + 1]);
            if (ray_hits_voxel(org, dir, cur[2 * i], p, l))
                total += (l < target) ? __builtin_popcount(octree[off0 + cur[2 * i + 1]]) : 1;
        }
        if (total > cap) {
            free(cur);
            return -1;
        }
        int32_t *nxt = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)(total > 0 ? total : 1));
        int64_t w = 0;
        for (int64_t i = 0; i < num; ++i) {
            const int32_t r = cur[2 * i], pid = cur[2 * i + 1];
            const int16_t *p = points + 4 * (off0 + pid);
            if (!ray_hits_voxel(org, dir, r, p, l)) continue;
            if (l == target) {
                nxt[2 * w] = r;
                nxt[2 * w + 1] = pid;
                ++w;
                continue;
            }
            const unsigned o = octree[off0 + pid];
            const uint32_t s = prefix[off0 + pid];
            const int code = origin_octant(org, r, p, l);
            for (int k = 0; k < 8; ++k) {
                const int j = child_order(code, k);
                if (o & (1u << j)) {
                    const unsigned cnt = (unsigned)__builtin_popcount(o & ((2u << j) - 1u));
                    nxt[2 * w] = r;
                    nxt[2 * w + 1] = (int32_t)((int64_t)s + cnt - off1);
                    ++w;
                }
            }
        }
        free(cur);
        cur = nxt;
        num = total;
        if (num == 0) break;
    }
    memcpy(out, cur, sizeof(int32_t) * 2 * (size_t)num);
    free(cur);
    return num;
}
