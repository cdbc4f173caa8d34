// Signed distance of points to a triangle mesh (compute_sdf ->
// mesh2sdf.mesh2sdf_gpu, sdf-net/lib/torchgp/compute_sdf.py:26-40, the
// DualSDF-derived kernels of sdf-net/lib/extensions/mesh2sdf_cuda/
// mesh2sdf_kernel.cu:307-617).
//
// Algorithm (as published there): the distance is the minimum over all
// triangles of the point-triangle distance -- the distance to the plane when
// the point projects inside the triangle (all three edge half-space tests
// agree), else to the nearest edge segment.  The sign comes from 13 fixed
// lines through the point (3 axes, 6 face diagonals, 4 body diagonals):
// the point is inside when every line crosses the mesh on both sides of it
// (Moller-Trumbore, |det| >= 1e-8), and the distance is then negated.
//
// GB300 layout: a per-triangle record of 92 floats is precomputed once: the
// three vertices, the three edge vectors, the normal, the three edge x
// normal vectors, the reciprocal squared lengths, for each of the 13 lines
// the point-independent part of the crossing test (pvec = dir x edge2 and
// 1/det, 0 where |det| < 1e-8), and a bounding sphere.  The distance kernel
// stages 128 records at a time in shared memory and every thread tests its
// point against them, keeping the running minimum and two 13-bit crossing
// masks in registers.  The sphere culls without changing any result: a
// triangle whose sphere lies farther than the running minimum cannot lower
// it, and a line that misses the sphere cannot cross the triangle (both
// tests with a relative margin far above float rounding).
#include "common.cuh"

namespace nglod {

constexpr int kTriRec = 92;      // floats per triangle record (368 bytes)
constexpr int kRecSphere = 88;   // bounding sphere: centre x y z, radius
constexpr int kRecInvDet = 36;   // 1/det of the 13 lines
constexpr int kRecPvec = 49;     // pvec of the 13 lines
constexpr int kTriTile = 128;    // triangles per shared-memory tile

__device__ __forceinline__ float dot3(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

__device__ __forceinline__ void cross3(const float *a, const float *b, float *r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

// |a x - b|^2
__device__ __forceinline__ float d2axmb(const float *a, float x, const float *b) {
    const float t0 = a[0] * x - b[0], t1 = a[1] * x - b[1], t2 = a[2] * x - b[2];
    return t0 * t0 + t1 * t1 + t2 * t2;
}

__constant__ float c_stab_dirs[13][3];
static const float h_stab_dirs[13][3] = {
    {1.f, 0.f, 0.f},
    {0.f, 1.f, 0.f},
    {0.f, 0.f, 1.f},
    {0.f, 0.707106781f, 0.707106781f},
    {0.707106781f, 0.f, 0.707106781f},
    {0.707106781f, 0.707106781f, 0.f},
    {0.f, 0.707106781f, -0.707106781f},
    {0.707106781f, 0.f, -0.707106781f},
    {0.707106781f, -0.707106781f, 0.f},
    {0.577350269f, 0.577350269f, 0.577350269f},
    {-0.577350269f, 0.577350269f, 0.577350269f},
    {0.577350269f, -0.577350269f, 0.577350269f},
    {0.577350269f, 0.577350269f, -0.577350269f},
};

// record: v0[0..2] v10[3..5] v21[6..8] v02[9..11] nor[12..14] c10[15..17]
// c21[18..20] c02[21..23] i10 i21 i02 inor [24..27] v1[28..30] v2[31..33]
// pad[34..35] inv_det[36..48] pvec[49..87] sphere[88..91]
__global__ void mesh_prepare_kernel(const float *__restrict__ tri, int64_t m, float *__restrict__ rec) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        const float *t = tri + 9 * i;
        float *r = rec + kTriRec * i;
        float v10[3], v21[3], v02[3], nor[3];
        for (int k = 0; k < 3; ++k) {
            v10[k] = t[3 + k] - t[k];
            v21[k] = t[6 + k] - t[3 + k];
            v02[k] = t[k] - t[6 + k];
        }
        cross3(v10, v02, nor);
        for (int k = 0; k < 3; ++k) {
            r[k] = t[k];
            r[3 + k] = v10[k];
            r[6 + k] = v21[k];
            r[9 + k] = v02[k];
            r[12 + k] = nor[k];
        }
        cross3(v10, nor, r + 15);
        cross3(v21, nor, r + 18);
        cross3(v02, nor, r + 21);
        r[24] = __fdiv_rn(1.f, dot3(v10, v10));
        r[25] = __fdiv_rn(1.f, dot3(v21, v21));
        r[26] = __fdiv_rn(1.f, dot3(v02, v02));
        r[27] = __fdiv_rn(1.f, dot3(nor, nor));
        for (int k = 0; k < 3; ++k) {
            r[28 + k] = t[3 + k];
            r[31 + k] = t[6 + k];
        }
        r[34] = r[35] = 0.f;
        const float e2v[3] = {-v02[0], -v02[1], -v02[2]};
        for (int d = 0; d < 13; ++d) {
            float pv[3];
            cross3(c_stab_dirs[d], e2v, pv);
            const float det = dot3(v10, pv);
            r[kRecInvDet + d] = (det > -1e-8f && det < 1e-8f) ? 0.f : __fdiv_rn(1.f, det);
            for (int k = 0; k < 3; ++k) r[kRecPvec + 3 * d + k] = pv[k];
        }
        // bounding sphere about the centroid, radius rounded up
        float c[3], rad2 = 0.f;
        for (int k = 0; k < 3; ++k) c[k] = (t[k] + t[3 + k] + t[6 + k]) * (1.f / 3.f);
        for (int v = 0; v < 3; ++v) {
            float d2 = 0.f;
            for (int k = 0; k < 3; ++k) d2 = fmaf(t[3 * v + k] - c[k], t[3 * v + k] - c[k], d2);
            rad2 = fmaxf(rad2, d2);
        }
        for (int k = 0; k < 3; ++k) r[kRecSphere + k] = c[k];
        r[kRecSphere + 3] = sqrtf(rad2) * 1.0001f + 1e-7f;
    }
}


__global__ void __launch_bounds__(kTriTile) mesh_sdf_kernel(const float *__restrict__ rec, int64_t m,
                                                            const float *__restrict__ pts, int64_t n,
                                                            float *__restrict__ out) {
    __shared__ float s[kTriTile * kTriRec];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // every thread of the block runs the same number of tile rounds
    const int64_t rounds = (n + stride - 1) / stride;
    for (int64_t rd = 0; rd < rounds; ++rd) {
        const int64_t i = rd * stride + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const bool valid = i < n;
        float p[3] = {0.f, 0.f, 0.f};
        if (valid) {
            p[0] = pts[3 * i];
            p[1] = pts[3 * i + 1];
            p[2] = pts[3 * i + 2];
        }
        float mind2 = INFINITY, mind = INFINITY;
        uint32_t pos = 0u, neg = 0u;
        for (int64_t t0 = 0; t0 < m; t0 += kTriTile) {
            const int cnt = (int)(m - t0 < kTriTile ? m - t0 : kTriTile);
            __syncthreads();
            for (int k = threadIdx.x; k < cnt * kTriRec / 4; k += blockDim.x)
                reinterpret_cast<float4 *>(s)[k] = reinterpret_cast<const float4 *>(rec + t0 * kTriRec)[k];
            __syncthreads();
            if (!valid) continue;
            for (int j = 0; j < cnt; ++j) {
                const float *r = s + j * kTriRec;
                float p0[3], p1[3], p2[3];
                for (int k = 0; k < 3; ++k) {
                    p0[k] = p[k] - r[k];
                    p1[k] = p[k] - r[28 + k];
                    p2[k] = p[k] - r[31 + k];
                }
                const float *v10 = r + 3, *v21 = r + 6, *v02 = r + 9, *nor = r + 12;
                const float w[3] = {r[kRecSphere] - p[0], r[kRecSphere + 1] - p[1], r[kRecSphere + 2] - p[2]};
                const float w2 = dot3(w, w), rho = r[kRecSphere + 3];
                const float reach = mind + rho;
                if ((nor[0] != 0.f || nor[1] != 0.f || nor[2] != 0.f) && !(w2 > reach * reach * 1.0001f)) {
                    const float s1 = copysignf(1.f, dot3(r + 15, p0));
                    const float s2 = copysignf(1.f, dot3(r + 18, p1));
                    const float s3 = copysignf(1.f, dot3(r + 21, p2));
                    float d2;
                    if (s1 + s2 + s3 < 2.f) {
                        const float e1 = d2axmb(v10, fmaxf(0.f, fminf(dot3(v10, p0) * r[24], 1.f)), p0);
                        const float e2 = d2axmb(v21, fmaxf(0.f, fminf(dot3(v21, p1) * r[25], 1.f)), p1);
                        const float e3 = d2axmb(v02, fmaxf(0.f, fminf(dot3(v02, p2) * r[26], 1.f)), p2);
                        d2 = fminf(e1, fminf(e2, e3));
                    } else {
                        const float dn = dot3(nor, p0);
                        d2 = dn * dn * r[27];
                    }
                    const float m2 = fminf(mind2, fmaxf(d2, 0.f));
                    if (m2 < mind2) {
                        mind2 = m2;
                        mind = __fsqrt_ru(m2);
                    }
                }
                // crossings of the 13 lines: edge1 = v10, edge2 = -v02, tvec = p0.
                // squared distance of a line from the centre is w2 - (w.d)^2, which
                // cancels: the margin covers its rounding (a few 1e-7 of w2)
                const float rho2 = fmaf(rho * rho, 1.0001f, fmaf(w2, 2e-6f, 1e-12f));
                const float e2v[3] = {-v02[0], -v02[1], -v02[2]};
                float qvec[3];
                cross3(p0, v10, qvec);
                const float qe2 = dot3(e2v, qvec);
#pragma unroll
                for (int d = 0; d < 13; ++d) {
                    const float inv_det = r[kRecInvDet + d];
                    if (inv_det == 0.f) continue;
                    const float *dir = c_stab_dirs[d];
                    const float wd = dot3(w, dir);
                    if (w2 - wd * wd > rho2) continue;  // the line misses the sphere
                    const float *pvec = r + kRecPvec + 3 * d;
                    const float u = dot3(p0, pvec) * inv_det;
                    if (u < 0.f || u > 1.f) continue;
                    const float v = dot3(dir, qvec) * inv_det;
                    if (v < 0.f || u + v > 1.f) continue;
                    const float tt = qe2 * inv_det;
                    if (tt >= 0.f)
                        pos |= 1u << d;
                    else
                        neg |= 1u << d;
                }
            }
        }
        if (valid) {
            const float dist = __fsqrt_rn(fmaxf(mind2, 0.f));
            const bool inside = (pos & neg) == 0x1FFFu;
            out[i] = inside ? -dist : dist;
        }
    }
}

}  // namespace nglod

using namespace nglod;

extern "C" int64_t nglod_mesh_record_floats(void) { return kTriRec; }

static int upload_stab_dirs() {
    static bool done[64] = {false};
    int dev = 0;
    NGLOD_TRY(cuda_status(cudaGetDevice(&dev), "mesh device"));
    NGLOD_REQUIRE(dev >= 0 && dev < 64, NGLOD_ERR_UNSUPPORTED, "device %d", dev);
    if (!done[dev]) {
        NGLOD_TRY(cuda_status(cudaMemcpyToSymbol(c_stab_dirs, h_stab_dirs, sizeof(h_stab_dirs)), "mesh dirs"));
        done[dev] = true;
    }
    return NGLOD_OK;
}

extern "C" int nglod_mesh_prepare(const float *triangles, int64_t m, float *records, nglod_stream_t stream) {
    NGLOD_REQUIRE(m >= 0, NGLOD_ERR_INVALID, "m=%lld is negative", (long long)m);
    if (m == 0) return NGLOD_OK;
    NGLOD_REQUIRE(triangles && records, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(aligned(records, 16), NGLOD_ERR_ALIGN, "records must be 16-byte aligned");
    NGLOD_TRY(upload_stab_dirs());
    const int64_t want = (m + 255) / 256, cap = (int64_t)num_sms() * 8;
    mesh_prepare_kernel<<<(int)(want < cap ? want : cap), 256, 0, (cudaStream_t)stream>>>(triangles, m, records);
    return launch_status("nglod_mesh_prepare");
}

extern "C" int nglod_mesh_sdf(const float *records, int64_t m, const float *points, int64_t n, float *out,
                              nglod_stream_t stream) {
    NGLOD_REQUIRE(m >= 0 && n >= 0, NGLOD_ERR_INVALID, "m=%lld, n=%lld", (long long)m, (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(points && out && (records || m == 0), NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(m == 0 || aligned(records, 16), NGLOD_ERR_ALIGN, "records must be 16-byte aligned");
    NGLOD_TRY(upload_stab_dirs());
    const int64_t want = (n + kTriTile - 1) / kTriTile, cap = (int64_t)num_sms() * 16;
    mesh_sdf_kernel<<<(int)(want < cap ? want : cap), kTriTile, 0, (cudaStream_t)stream>>>(records, m, points, n,
                                                                                        out);
    return launch_status("nglod_mesh_sdf");
}
