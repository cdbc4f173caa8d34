/*
 * nglod_gb300.h -- C ABI of the GB300-native NGLOD neural-SDF hot path.
 *
 * Every entry point takes raw device pointers, int64 sizes and a CUDA stream,
 * launches asynchronously on that stream, never allocates or frees caller
 * memory, never synchronises the device, and returns NGLOD_OK (0) or a
 * negative status.  The message of the last failure on the calling host
 * thread is returned by nglod_last_error().  No C++ exception crosses this
 * boundary.
 *
 * Data layout shared by all entry points:
 *   points / ray origins / ray directions   float32 [n][3], 4-byte aligned
 *   feature volume i (dense model)          channel-last [s][s][s][C] with
 *       s = 2^(i + base_lod) + 1 vertices per side, index ((z*s + y)*s + x)*C + c,
 *       x = the W axis of the reference's fm[1, C, D, H, W]; 16-byte aligned
 *   decoder i                               w0 [H][3+C], b0 [H], w1 [H], b1 [1]
 *       (nn.Linear layouts of louts[i][0] and louts[i][2])
 */
#ifndef NGLOD_GB300_H
#define NGLOD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *nglod_stream_t; /* same type as cudaStream_t */

#define NGLOD_OK               0
#define NGLOD_ERR_INVALID     -1  /* bad argument: null pointer, size, shape */
#define NGLOD_ERR_UNSUPPORTED -2  /* configuration not built (e.g. feature_dim) */
#define NGLOD_ERR_CUDA        -3  /* CUDA runtime error at launch */
#define NGLOD_ERR_CAPACITY    -4  /* output capacity exceeded */
#define NGLOD_ERR_ALIGN       -5  /* pointer alignment requirement not met */
#define NGLOD_ERR_TIMEOUT     -6  /* bounded device wait gave up */

#define NGLOD_MAX_LODS 8

#define NGLOD_F32  0
#define NGLOD_BF16 1

/* A dense OctreeSDF: num_lods feature volumes and one decoder per LOD.
 * Mirrors OctreeSDF.__init__ (sdf-net/lib/models/OctreeSDF.py:60-88). */
typedef struct nglod_dense_model {
    int32_t num_lods;      /* 1..NGLOD_MAX_LODS */
    int32_t base_lod;      /* volume i has 2^(i+base_lod)+1 vertices per side */
    int32_t feature_dim;   /* C; 32 is built */
    int32_t hidden_dim;    /* H; 1..256 */
    int32_t grid_dtype;    /* NGLOD_F32 (bf16 volumes: see nglod_sdf_fwd_bf16) */
    int32_t reserved;
    const void  *grid[NGLOD_MAX_LODS];
    const float *w0[NGLOD_MAX_LODS];
    const float *b0[NGLOD_MAX_LODS];
    const float *w1[NGLOD_MAX_LODS];
    const float *b1[NGLOD_MAX_LODS];
} nglod_dense_model;

/* SphereTracer settings (sdf-net/lib/tracer/BaseTracer.py:29-45,
 * sdf-net/lib/options.py:209-221). */
typedef struct nglod_trace_params {
    int32_t num_steps;     /* march iterations (reference default 256) */
    float   min_dis;       /* |d| > min_dis keeps a ray marching (3e-4) */
    float   osc_dis;       /* |(d+dprev)/2| > osc_dis keeps it marching (3*min_dis) */
    float   step_size;     /* scale of each step (1.0) */
    float   far_clip;      /* |t| < far_clip keeps it marching: camera_clamp[1] (10.0) */
    int32_t lod;           /* LOD of every sdf evaluation; <0 or >=num_lods: finest */
    int32_t want_normals;  /* 1: finite-difference normals of hit rays */
} nglod_trace_params;

const char *nglod_version(void);
const char *nglod_last_error(void);

/* Ray vs the [-1,1]^3 box.  Replaces sol_nglod.aabb
 * (sdf-net/lib/extensions/sol_nglod/sol_nglod_kernel.cu:161-188, kernel 77-159).
 * Writes every output element: x = entry point (ray_o where missed or where
 * the origin is inside the box), t = entry distance (0 where not hit),
 * hit = 1/0.  Bit-exact with the reference kernel's float arithmetic. */
int nglod_aabb(const float *ray_o, const float *ray_d, int64_t n,
               float *x, float *t, uint8_t *hit, nglod_stream_t stream);

/* One channel-last float32 feature volume (side^3 vertices, feature_dim
 * channels) sampled trilinearly at n points: out[n][feature_dim].  Replaces
 * FeatureVolume.forward (sdf-net/lib/models/OctreeSDF.py:46-57), i.e.
 * F.grid_sample(align_corners=True, padding_mode='border').  grid and out
 * 16-byte aligned. */
int nglod_volume_sample(const float *grid, int32_t side, int32_t feature_dim, const float *x, int64_t n,
                        float *out, nglod_stream_t stream);

/* Fused per-LOD trilinear gather + running sum + decoder, float32.
 * Replaces OctreeSDF.sdf(x, lod, return_lst) (OctreeSDF.py:94-155) and
 * BaseLOD.forward (sdf-net/lib/models/BaseLOD.py:37-41).
 * lod in [0, num_lods): out[n] = prediction of that LOD;
 * lod < 0 or >= num_lods: the finest prediction;
 * all_lods != 0: out[num_lods][n] = every LOD's prediction (return_lst). */
int nglod_sdf_fwd(const nglod_dense_model *model, const float *x, int64_t n,
                  int32_t lod, int32_t all_lods, float *out, nglod_stream_t stream);

/* Persistent fused sphere tracer, float32: aabb prologue, march loop,
 * AABB cull and finite-difference normals in one launch.  Replaces
 * SphereTracer.forward (sdf-net/lib/tracer/SphereTracer.py:41-132) with
 * gradient(method='finitediff') (sdf-net/lib/diffutils.py:61-70).
 * work_counter: one device int64 used to hand rays to warps; the call zeroes
 * it on the stream before the launch.  Outputs x[n][3], t[n], hit[n],
 * normal[n][3] are all written. */
int nglod_trace(const nglod_dense_model *model, const nglod_trace_params *params,
                const float *ray_o, const float *ray_d, int64_t n,
                float *x, float *t, uint8_t *hit, float *normal,
                int64_t *work_counter, nglod_stream_t stream);

/* ------------------------------------------------------------------------
 * Training: forward with saved features, hand-written backward, Adam.
 * ------------------------------------------------------------------------ */

/* Gradient buffers of a dense model, same layouts as the parameters
 * (volumes channel-last).  Backward ADDS into them, as autograd accumulates
 * into .grad; callers zero them first. */
typedef struct nglod_dense_grads {
    float *grid[NGLOD_MAX_LODS];
    float *w0[NGLOD_MAX_LODS];
    float *b0[NGLOD_MAX_LODS];
    float *w1[NGLOD_MAX_LODS];
    float *b1[NGLOD_MAX_LODS];
} nglod_dense_grads;

/* Forward of the LODs in lod_mask (bit l = LOD l) for training.  With
 * L = highest set bit: preds[l][n] and feats[l][n][C] (the running feature
 * sum that decoder l reads) are written for every l in the mask.  Same
 * predictions as OctreeSDF.sdf(x, lod=l) for each l in the mask
 * (OctreeSDF.py:94-146); with all bits set, as sdf(x, return_lst=True). */
int nglod_sdf_fwd_train(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                        float *preds, float *feats, nglod_stream_t stream);

/* Backward of nglod_sdf_fwd_train.  grad_preds[l][n] = dLoss/dpred_l for l in
 * lod_mask.  Adds the parameter gradients into `grads` and, when grad_x is
 * not NULL, dLoss/dx into grad_x[n][3].  dfeat_scratch[L+1][n][C] is caller-
 * provided scratch.  Replaces the autograd backward of OctreeSDF.sdf through
 * nn.Linear and F.grid_sample (border padding, align_corners) that
 * Trainer.step_geometry runs (sdf-net/lib/trainer.py:339): decoder weight
 * gradients are per-block tile reductions, feature gradients a trilinear
 * scatter-add (coarse volumes accumulated in shared memory, the rest with
 * vector atomics). */
int nglod_sdf_bwd(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                  const float *grad_preds, const float *feats, float *dfeat_scratch,
                  const nglod_dense_grads *grads, float *grad_x, nglod_stream_t stream);

/* nglod_sdf_bwd for callers that cannot allocate device memory (a plugin
 * whose GPU memory is owned by its host application, a process whose
 * allocator is locked after start-up): the same backward, but the per-point
 * scratch comes from a fixed array inside the library instead of a
 * caller-provided buffer, and the call allocates nothing.  No counterpart in
 * the reference.
 * Limit: (highest LOD in lod_mask + 1) * n * feature_dim floats must fit in
 * NGLOD_NOALLOC_SCRATCH_BYTES (16 MiB on every GPU that loads the library,
 * held until exit): n <= 26,214 with 5 LODs, 131,072 with one; larger n
 * returns NGLOD_ERR_CAPACITY.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller. */
#define NGLOD_NOALLOC_SCRATCH_BYTES (16u << 20)
int nglod_sdf_bwd_noalloc(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                          const float *grad_preds, const float *feats, const nglod_dense_grads *grads,
                          float *grad_x, nglod_stream_t stream);

/* One tensor of a multi-tensor Adam step (device-resident table). */
typedef struct nglod_adam_tensor {
    float       *param;
    const float *grad;
    float       *exp_avg;
    float       *exp_avg_sq;
    int64_t      numel;
} nglod_adam_tensor;

/* Adam update of `count` tensors described by the device table `tensors`,
 * step = the step number after increment (1 for the first step).  Same
 * update order as torch.optim.Adam's single-tensor path with amsgrad=False,
 * maximize=False (the optimizer of sdf-net/lib/trainer.py:184-185):
 * m = lerp(m, g, 1-beta1); v = v*beta2 + (1-beta2)*g*g;
 * p -= lr/(1-beta1^step) * m / (sqrt(v)/sqrt(1-beta2^step) + eps).
 * weight_decay adds weight_decay*p to g first (0 in the reference). */
int nglod_adam_step(const nglod_adam_tensor *tensors, int32_t count, int64_t max_numel, float lr, float beta1,
                    float beta2, float eps, float weight_decay, int64_t step, nglod_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* NGLOD_GB300_H */
