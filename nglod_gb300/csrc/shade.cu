// Shading passes on a traced render buffer: the reference Renderer's ground
// plane and shadow rays, ambient occlusion, relative depth, matcap lookup,
// shadow-map blur and compositing (sdf-net/lib/renderer.py:118-223,
// sdf-net/lib/geoutils.py:237-276).  Every pass writes a device buffer; no
// graphics API is involved.
//
// Float arithmetic follows the reference's torch expressions one operation
// at a time (no contraction): a torch product then sum is __fmul_rn then
// __fadd_rn here.
#include <math.h>

#include "common.cuh"
#include "scan.cuh"

namespace nglod {

constexpr int kAoTaps = 40;

inline int shade_grid(int64_t n, int threads = 256) {
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)num_sms() * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Lowest y of the hit points (the reference takes the ground height from the
// lowest surface sample, renderer.py:76-86); +inf when nothing was hit.
__global__ void min_hit_y_kernel(const float *__restrict__ x, const uint8_t *__restrict__ hit, int64_t n,
                                 unsigned int *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    float m = INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (hit[i]) m = fminf(m, x[3 * i + 1]);
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    // order-preserving map of floats to unsigned ints for atomicMin
    if ((threadIdx.x & 31) == 0) {
        const unsigned int u = __float_as_uint(m);
        atomicMin(out, (u & 0x80000000u) ? ~u : (u | 0x80000000u));
    }
}

// Ground plane y = min_y (renderer.py:131-150): rays that reach the plane
// before their surface hit take the plane's depth, position and normal
// (0, 1, 0) and stop being surface hits.
__global__ void ground_kernel(const float *__restrict__ ro, const float *__restrict__ rd, int64_t n, float min_y,
                              float *x, float *t, uint8_t *hit, float *normal, uint8_t *plane_hit) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float rate = -rd[3 * i + 1];
        const float delta = __fsub_rn(ro[3 * i + 1], min_y);
        const float pt = __fdiv_rn(delta, rate);
        const bool ph = (pt > 0.f) && (pt < 500.f) && (pt < t[i]);
        plane_hit[i] = ph ? 1 : 0;
        if (ph) {
            hit[i] = 0;
            t[i] = pt;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                x[3 * i + k] = __fadd_rn(ro[3 * i + k], __fmul_rn(rd[3 * i + k], pt));
                normal[3 * i + k] = k == 1 ? 1.f : 0.f;
            }
        }
    }
}

// Shadow rays (renderer.py:152-161): origin x + 0.1 n, direction towards the
// light with the caller's N(0, 0.01^2) noise, normalised as F.normalize
// (eps 1e-12); light_hit = the direction faces the normal's side.
__global__ void shadow_rays_kernel(const float *__restrict__ x, const float *__restrict__ normal,
                                   const float *__restrict__ noise, int64_t n, float lx, float ly, float lz,
                                   float *so, float *sd, uint8_t *light_hit) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const float light[3] = {lx, ly, lz};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float o[3], d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            o[k] = __fadd_rn(x[3 * i + k], __fmul_rn(0.1f, normal[3 * i + k]));
            d[k] = __fsub_rn(__fadd_rn(noise[3 * i + k], light[k]), o[k]);
        }
        const float ss = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
        const float nrm = fmaxf(__fsqrt_rn(ss), 1e-12f);
        float dn = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            d[k] = __fdiv_rn(d[k], nrm);
            so[3 * i + k] = o[k];
            sd[3 * i + k] = d[k];
        }
        dn = __fadd_rn(__fadd_rn(__fmul_rn(d[0], normal[3 * i]), __fmul_rn(d[1], normal[3 * i + 1])),
                       __fmul_rn(d[2], normal[3 * i + 2]));
        light_hit[i] = dn > 0.f ? 1 : 0;
    }
}

// Ambient occlusion (renderer.py:184-208): 40 taps q_i = x + n * d_i along the
// normal with d_i = 0.025 ((i+1)/41)^1.6, evaluated by the caller's sdf call.
// Rays shaded are the surface hits and (with shadows) the ground-plane hits.
__global__ void ao_flag_chunk_kernel(const uint8_t *__restrict__ hit, const uint8_t *__restrict__ plane_hit,
                                     const int64_t *count, uint32_t *partials) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && (hit[i] || (plane_hit && plane_hit[i]))) ? 1u : 0u;
        const uint32_t s = block_sum(f, s_warp);
        if (threadIdx.x == 0) partials[c] = s;
    }
}

__global__ void ao_emit_kernel(const uint8_t *__restrict__ hit, const uint8_t *__restrict__ plane_hit,
                               const int64_t *count, const uint32_t *__restrict__ partials, int32_t *idx) {
    __shared__ uint32_t s_warp[33];
    const int64_t n = *count;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t i = c * kChunk + threadIdx.x;
        const uint32_t f = (i < n && (hit[i] || (plane_hit && plane_hit[i]))) ? 1u : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(f, s_warp, &tot);
        if (f) idx[partials[c] + ex] = (int32_t)i;
    }
}

__constant__ float c_ao_d[kAoTaps];

__global__ void ao_taps_kernel(const float *__restrict__ x, const float *__restrict__ normal,
                               const int32_t *__restrict__ idx, int64_t m, float *taps) {
    const int64_t total = m * kAoTaps;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += stride) {
        const int64_t j = k / kAoTaps;
        const int tap = (int)(k - j * kAoTaps);
        const int64_t i = idx[j];
        const float d = c_ao_d[tap];
#pragma unroll
        for (int c = 0; c < 3; ++c) taps[3 * k + c] = __fadd_rn(x[3 * i + c], __fmul_rn(normal[3 * i + c], d));
    }
}

// acc over the taps in order: acc += 3.5 relu(d - r - 0.0015), where a
// ground-plane ray's r is min(sdf, d); ao = clamp(1 - acc, 0.1, 1)^2, and 1
// for rays that are not shaded.
__global__ void ao_reduce_kernel(const float *__restrict__ r, const int32_t *__restrict__ idx, int64_t m,
                                 const uint8_t *__restrict__ plane_hit, float *ao) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) {
        const int64_t i = idx[j];
        const bool plane = plane_hit && plane_hit[i];
        float acc = 0.f;
        for (int tap = 0; tap < kAoTaps; ++tap) {
            const float d = c_ao_d[tap];
            float v = r[j * kAoTaps + tap];
            if (plane) v = fminf(v, d);
            const float e = __fsub_rn(__fsub_rn(d, v), 0.0015f);
            acc = __fadd_rn(acc, __fmul_rn(3.5f, fmaxf(e, 0.f)));
        }
        float a = fminf(fmaxf(__fsub_rn(1.f, acc), 0.1f), 1.f);
        ao[i] = __fmul_rn(a, a);
    }
}

__global__ void fill_kernel(float *p, int64_t n, float v) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

// Matcap colour (renderer.py:262-279, geoutils.py:253-276): the reflected
// view direction gives texture coordinates vN in [0,1]^2, sampled
// bilinearly from the texture (rows along the first coordinate, as the
// reference's interpolator over the transposed image); hit pixels only, the
// others are white.  texture: float32 [tex_w][tex_h][3] (0..255).
__global__ void matcap_kernel(const float *__restrict__ view, const float *__restrict__ normal,
                              const uint8_t *__restrict__ hit, int64_t n, const float *__restrict__ tex, int tw,
                              int th, float *rgb) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (!hit[i]) {
            rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = 1.f;
            continue;
        }
        const float v0 = view[3 * i], v1 = view[3 * i + 1], v2 = -view[3 * i + 2];
        const float n0 = normal[3 * i], n1 = normal[3 * i + 1], n2 = normal[3 * i + 2];
        const float dot = __fadd_rn(__fadd_rn(__fmul_rn(n0, v0), __fmul_rn(n1, v1)), __fmul_rn(n2, v2));
        const float two_dot = __fmul_rn(2.f, dot);
        const float r0 = __fsub_rn(v0, __fmul_rn(two_dot, n0));
        const float r1 = __fsub_rn(v1, __fmul_rn(two_dot, n1));
        const float r2 = __fsub_rn(__fsub_rn(v2, __fmul_rn(two_dot, n2)), 1.f);
        const float ss = __fadd_rn(__fadd_rn(__fmul_rn(r0, r0), __fmul_rn(r1, r1)), __fmul_rn(r2, r2));
        const float mm = __fmul_rn(2.f, __fsqrt_rn(ss));
        float u = __fsub_rn(1.f, __fadd_rn(__fdiv_rn(r0, mm), 0.5f));
        float v = __fsub_rn(1.f, __fadd_rn(__fdiv_rn(r1, mm), 0.5f));
        u = isnan(u) ? 0.f : fminf(fmaxf(u, 0.f), 1.f);
        v = isnan(v) ? 0.f : fminf(fmaxf(v, 0.f), 1.f);
        // grid points k / (size - 1): cell and fraction along each axis
        const float fu = u * (float)(tw - 1), fv = v * (float)(th - 1);
        int iu = min((int)fu, tw - 2), iv = min((int)fv, th - 2);
        iu = max(iu, 0);
        iv = max(iv, 0);
        const float au = fu - (float)iu, av = fv - (float)iv;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float t00 = tex[((int64_t)iu * th + iv) * 3 + c], t01 = tex[((int64_t)iu * th + iv + 1) * 3 + c];
            const float t10 = tex[((int64_t)(iu + 1) * th + iv) * 3 + c];
            const float t11 = tex[((int64_t)(iu + 1) * th + iv + 1) * 3 + c];
            const float a = t00 + (t01 - t00) * av, b = t10 + (t11 - t10) * av;
            rgb[3 * i + c] = (a + (b - a) * au) / 255.f;
        }
    }
}

// Separable Gaussian (scipy.ndimage.gaussian_filter, mode 'reflect',
// truncate 4): one axis of a [rows][cols] float image, summed in double as a
// symmetric filter (centre tap, then the pairs in[-o] + in[+o] times w[o]),
// each pass rounded to float as scipy's float32 output is.  axis 0 runs down
// the rows.  c_gauss[o] = normalised weight of offset o >= 0.
__constant__ double c_gauss[17];
__device__ __forceinline__ int reflect_index(int p, int len) {
    // 'reflect': d c b a | a b c d | d c b a
    while (p < 0 || p >= len) p = p < 0 ? -p - 1 : 2 * len - p - 1;
    return p;
}
__global__ void blur_axis_kernel(const float *__restrict__ in, float *out, int rows, int cols, int axis, int radius) {
    const int64_t n = (int64_t)rows * cols;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const int r = (int)(k / cols), c = (int)(k - (int64_t)r * cols);
        const int len = axis == 0 ? rows : cols;
        const int pos = axis == 0 ? r : c;
        auto at = [&](int p) -> double {
            p = reflect_index(p, len);
            return (double)(axis == 0 ? in[(int64_t)p * cols + c] : in[(int64_t)r * cols + p]);
        };
        double s = at(pos) * c_gauss[0];
        for (int o = 1; o <= radius; ++o) s += (at(pos - o) + at(pos + o)) * c_gauss[o];
        out[k] = (float)s;
    }
}

// rgb *= (shadow ? blurred shadow map : 1) * (ao ? ao : 1); the shadow map
// before the blur is clamp(1 - shadow + 0.9, 0, 1).
__global__ void shadow_map_kernel(const uint8_t *__restrict__ shadow_hit, const uint8_t *__restrict__ light_hit,
                                  int64_t n, float *map, uint8_t *shadow) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const bool s = shadow_hit[i] && light_hit[i];
        shadow[i] = s ? 1 : 0;
        map[i] = fminf(fmaxf(__fadd_rn(__fsub_rn(1.f, s ? 1.f : 0.f), 0.9f), 0.f), 1.f);
    }
}

__global__ void compose_kernel(float *rgb, int64_t n, const float *__restrict__ smap, const float *__restrict__ ao,
                               const float *__restrict__ t, float far_clip, float *rel_depth) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (rgb) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v = rgb[3 * i + c];
                if (smap) v = __fmul_rn(v, smap[i]);
                if (ao) v = __fmul_rn(v, ao[i]);
                rgb[3 * i + c] = v;
            }
        }
        if (rel_depth) rel_depth[i] = __fdiv_rn(fminf(fmaxf(t[i], 0.f), far_clip), far_clip);
    }
}

}  // namespace nglod

using namespace nglod;

extern "C" int nglod_shade_min_hit_y(const float *x, const uint8_t *hit, int64_t n, uint32_t *out_key,
                                     nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0 && out_key, NGLOD_ERR_INVALID, "bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t init = 0xFFFFFFFFu;
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(out_key, &init, sizeof(init), cudaMemcpyHostToDevice, s), "min y init"));
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && hit, NGLOD_ERR_INVALID, "null pointer argument");
    min_hit_y_kernel<<<shade_grid(n), 256, 0, s>>>(x, hit, n, out_key);
    return launch_status("nglod_shade_min_hit_y");
}

extern "C" int nglod_shade_ground(const float *ray_o, const float *ray_d, int64_t n, float min_y, float *x, float *t,
                                  uint8_t *hit, float *normal, uint8_t *plane_hit, nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ray_o && ray_d && x && t && hit && normal && plane_hit, NGLOD_ERR_INVALID, "null pointer argument");
    ground_kernel<<<shade_grid(n), 256, 0, (cudaStream_t)stream>>>(ray_o, ray_d, n, min_y, x, t, hit, normal,
                                                                   plane_hit);
    return launch_status("nglod_shade_ground");
}

extern "C" int nglod_shade_shadow_rays(const float *x, const float *normal, const float *noise, int64_t n,
                                       const float *light_host, float *shadow_o, float *shadow_d, uint8_t *light_hit,
                                       nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0 && light_host, NGLOD_ERR_INVALID, "bad argument");
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && normal && noise && shadow_o && shadow_d && light_hit, NGLOD_ERR_INVALID,
                  "null pointer argument");
    shadow_rays_kernel<<<shade_grid(n), 256, 0, (cudaStream_t)stream>>>(
        x, normal, noise, n, light_host[0], light_host[1], light_host[2], shadow_o, shadow_d, light_hit);
    return launch_status("nglod_shade_shadow_rays");
}

extern "C" int nglod_shade_ao_select(const uint8_t *hit, const uint8_t *plane_hit, int64_t n, int32_t *idx,
                                     uint32_t *partials, int64_t *ctrl, int64_t *count, nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0 && count, NGLOD_ERR_INVALID, "bad argument");
    *count = 0;
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(hit && idx && partials && ctrl, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(n < ((int64_t)1 << 31), NGLOD_ERR_UNSUPPORTED, "n=%lld: ray indices are int32", (long long)n);
    NGLOD_REQUIRE(aligned(ctrl, 8), NGLOD_ERR_ALIGN, "ctrl must be 8-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(ctrl, &n, sizeof(int64_t), cudaMemcpyHostToDevice, s), "ao copy"));
    const int64_t chunks = (n + kChunk - 1) / kChunk;
    const int64_t cap = (int64_t)num_sms() * 2;
    const int grid = (int)(chunks < cap ? chunks : cap);
    ao_flag_chunk_kernel<<<grid, kChunk, 0, s>>>(hit, plane_hit, ctrl, partials);
    scan_chunk_counts_kernel<<<1, kChunk, 0, s>>>(partials, ctrl, ctrl + 1, INT64_MAX, nullptr);
    ao_emit_kernel<<<grid, kChunk, 0, s>>>(hit, plane_hit, ctrl, partials, idx);
    NGLOD_TRY(launch_status("nglod_shade_ao_select"));
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(count, ctrl + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "ao copy"));
    return cuda_status(cudaStreamSynchronize(s), "ao sync");
}

static int upload_ao_taps() {
    static bool done[64] = {false};
    int dev = 0;
    NGLOD_TRY(cuda_status(cudaGetDevice(&dev), "ao device"));
    NGLOD_REQUIRE(dev >= 0 && dev < 64, NGLOD_ERR_UNSUPPORTED, "device %d", dev);
    if (done[dev]) return NGLOD_OK;
    float d[kAoTaps];
    // the reference computes d_i in double and uses it against float32 tensors
    for (int i = 0; i < kAoTaps; ++i) d[i] = (float)(0.1 * 0.25 * pow((double)(i + 1) / (double)(kAoTaps + 1), 1.6));
    NGLOD_TRY(cuda_status(cudaMemcpyToSymbol(c_ao_d, d, sizeof(d)), "ao taps"));
    done[dev] = true;
    return NGLOD_OK;
}

extern "C" int nglod_shade_ao_taps(const float *x, const float *normal, const int32_t *idx, int64_t m, float *taps,
                                   nglod_stream_t stream) {
    NGLOD_REQUIRE(m >= 0, NGLOD_ERR_INVALID, "m=%lld is negative", (long long)m);
    if (m == 0) return NGLOD_OK;
    NGLOD_REQUIRE(x && normal && idx && taps, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_TRY(upload_ao_taps());
    ao_taps_kernel<<<shade_grid(m * kAoTaps), 256, 0, (cudaStream_t)stream>>>(x, normal, idx, m, taps);
    return launch_status("nglod_shade_ao_taps");
}

extern "C" int nglod_shade_ao_reduce(const float *r, const int32_t *idx, int64_t m, const uint8_t *plane_hit,
                                     int64_t n, float *ao, nglod_stream_t stream) {
    NGLOD_REQUIRE(m >= 0 && n >= 0 && m <= n, NGLOD_ERR_INVALID, "m=%lld, n=%lld", (long long)m, (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(ao && (m == 0 || (r && idx)), NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_TRY(upload_ao_taps());
    cudaStream_t s = (cudaStream_t)stream;
    fill_kernel<<<shade_grid(n), 256, 0, s>>>(ao, n, 1.f);
    if (m > 0) ao_reduce_kernel<<<shade_grid(m), 256, 0, s>>>(r, idx, m, plane_hit, ao);
    return launch_status("nglod_shade_ao_reduce");
}

extern "C" int nglod_shade_matcap(const float *view, const float *normal, const uint8_t *hit, int64_t n,
                                  const float *texture, int32_t tex_w, int32_t tex_h, float *rgb,
                                  nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0 && tex_w >= 2 && tex_h >= 2, NGLOD_ERR_INVALID, "n=%lld, texture %dx%d", (long long)n,
                  tex_w, tex_h);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE(view && normal && hit && texture && rgb, NGLOD_ERR_INVALID, "null pointer argument");
    matcap_kernel<<<shade_grid(n), 256, 0, (cudaStream_t)stream>>>(view, normal, hit, n, texture, tex_w, tex_h, rgb);
    return launch_status("nglod_shade_matcap");
}

extern "C" int nglod_shade_shadow_map(const uint8_t *shadow_hit, const uint8_t *light_hit, int32_t rows,
                                      int32_t cols, float sigma, float *map, float *scratch, uint8_t *shadow,
                                      nglod_stream_t stream) {
    NGLOD_REQUIRE(rows >= 1 && cols >= 1 && sigma > 0.f, NGLOD_ERR_INVALID, "image %dx%d, sigma %g", rows, cols,
                  (double)sigma);
    NGLOD_REQUIRE(shadow_hit && light_hit && map && scratch && shadow, NGLOD_ERR_INVALID, "null pointer argument");
    const int radius = (int)(4.0 * (double)sigma + 0.5);
    NGLOD_REQUIRE(radius <= 16, NGLOD_ERR_UNSUPPORTED, "sigma %g: Gaussian radius %d > 16", (double)sigma, radius);
    // exp(-x^2 / (2 sigma^2)) over x = -radius .. radius, normalised by the sum
    // taken in that order (scipy's _gaussian_kernel1d)
    double w[33], sum = 0.0;
    const double sig = (double)sigma;
    for (int o = -radius; o <= radius; ++o) {
        w[o + radius] = exp(-0.5 / (sig * sig) * (double)(o * o));
        sum += w[o + radius];
    }
    double half[17];
    for (int o = 0; o <= radius; ++o) half[o] = w[radius + o] / sum;
    cudaStream_t s = (cudaStream_t)stream;
    NGLOD_TRY(cuda_status(cudaMemcpyToSymbolAsync(c_gauss, half, sizeof(double) * (radius + 1), 0,
                                                  cudaMemcpyHostToDevice, s),
                          "gaussian weights"));
    const int64_t n = (int64_t)rows * cols;
    shadow_map_kernel<<<shade_grid(n), 256, 0, s>>>(shadow_hit, light_hit, n, map, shadow);
    blur_axis_kernel<<<shade_grid(n), 256, 0, s>>>(map, scratch, rows, cols, 0, radius);
    blur_axis_kernel<<<shade_grid(n), 256, 0, s>>>(scratch, map, rows, cols, 1, radius);
    return launch_status("nglod_shade_shadow_map");
}

extern "C" int nglod_shade_compose(float *rgb, int64_t n, const float *shadow_map, const float *ao, const float *t,
                                   float far_clip, float *relative_depth, nglod_stream_t stream) {
    NGLOD_REQUIRE(n >= 0, NGLOD_ERR_INVALID, "n=%lld is negative", (long long)n);
    if (n == 0) return NGLOD_OK;
    NGLOD_REQUIRE((rgb || relative_depth) && (!relative_depth || (t && far_clip > 0.f)), NGLOD_ERR_INVALID,
                  "bad argument");
    compose_kernel<<<shade_grid(n), 256, 0, (cudaStream_t)stream>>>(rgb, n, shadow_map, ao, t, far_clip,
                                                                    relative_depth);
    return launch_status("nglod_shade_compose");
}
