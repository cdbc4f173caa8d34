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
 * all_lods != 0: out[num_lods][n] = every LOD's prediction (return_lst).
 * Gathers and LOD sums are float32.  For one LOD at hidden_dim 128 a
 * persistent kernel (one block per SM, the leading volumes that fit copied
 * into shared memory) runs the decoder's first layer, features, x y z and
 * bias, on the tensor cores as split-TF32 products (relative error about
 * 2^-21 of the dot product, float32's own size); a bounded wait of that
 * kernel that gives up sets the flag nglod_dense_status reads.  Other shapes
 * decode per thread in float32. */
int nglod_sdf_fwd(const nglod_dense_model *model, const float *x, int64_t n,
                  int32_t lod, int32_t all_lods, float *out, nglod_stream_t stream);

/* nglod_sdf_fwd with the per-thread float32 decoder for every shape (the
 * tensor-core form is not used).  No counterpart in the reference: for
 * comparisons of the two forms. */
int nglod_sdf_fwd_simt(const nglod_dense_model *model, const float *x, int64_t n, int32_t lod, int32_t all_lods,
                       float *out, nglod_stream_t stream);

/* Reads and clears the float32 query's device status on the current device
 * (synchronous): *status_out = 1 if a bounded tensor-core wait of an
 * nglod_sdf_fwd or nglod_trace call since the last read gave up (its outputs
 * are incomplete), else 0.  No counterpart in the reference. */
int nglod_dense_status(int32_t *status_out);

/* nglod_sdf_fwd with the points and results in HOST memory: x_host [n][3],
 * out_host [n].  When both are pinned and mapped (cudaHostAlloc,
 * cudaHostRegister; PyTorch's pin_memory), one kernel launch reads the points
 * and writes the results over the host link itself.  Otherwise the points go
 * through a device staging area in chunks of `chunk` points; chunk i's copy
 * in, kernel and copy out run on one of three streams (the caller's and two
 * library streams forked from and joined back into it), so the copies of
 * one chunk overlap the kernels of the others.  scratch: device buffer of
 * nglod_host_query_scratch_bytes(chunk) bytes, 256-byte aligned.  Queued on
 * `stream` like every other call: out_host is complete when the work queued
 * on `stream` is; x_host, out_host and scratch must stay valid until then.
 * No reference counterpart (the reference takes device tensors only). */
int64_t nglod_host_query_scratch_bytes(int64_t chunk);
int nglod_sdf_fwd_host(const nglod_dense_model *model, const float *x_host, int64_t n, int32_t lod,
                       float *out_host, int64_t chunk, void *scratch, nglod_stream_t stream);

/* Persistent fused sphere tracer, float32: aabb prologue, march loop,
 * AABB cull and finite-difference normals in one launch.  Replaces
 * SphereTracer.forward (sdf-net/lib/tracer/SphereTracer.py:41-132) with
 * gradient(method='finitediff') (sdf-net/lib/diffutils.py:61-70).
 * work_counter: one device int64 used to hand rays to warps; the call zeroes
 * it on the stream before the launch.  Outputs x[n][3], t[n], hit[n],
 * normal[n][3] are all written.  At hidden_dim 128 every sdf evaluation is
 * nglod_sdf_fwd's tensor-core arithmetic (the same bits at the same point);
 * a bounded wait that gives up sets the flag nglod_dense_status reads. */
int nglod_trace(const nglod_dense_model *model, const nglod_trace_params *params,
                const float *ray_o, const float *ray_d, int64_t n,
                float *x, float *t, uint8_t *hit, float *normal,
                int64_t *work_counter, nglod_stream_t stream);

/* Pinhole camera rays of the reference's look_at (sdf-net/lib/geoutils.py:
 * 180-206, 'persp' mode) without the random pixel jitter of normalized_grid
 * (geoutils.py:149-152): origins = eye, unit directions, ray i = ix*height + iy.
 * eye/at/up are host float[3]. */
int nglod_camera_rays(const float *eye, const float *at, const float *up, float fov_deg, int32_t width,
                      int32_t height, float *org, float *dir, nglod_stream_t stream);

/* ------------------------------------------------------------------------
 * BF16 form: bf16 feature volumes and a tcgen05 tensor-core decoder.
 *
 * The decoder's first layer runs as a 128-point x 128-hidden x 48 bf16 tile
 * product with fp32 accumulation in tensor memory.  K order of the tile:
 * k 0..31 = the 32 summed features, 32..34 = x, y, z rounded to bf16,
 * 35..37 = the bf16 remainders x - bf16(x) (so positions keep ~16 bits),
 * 38, 39 = 1.0 against the bf16 split b0 = hi + lo of the first-layer bias,
 * 40..47 = 0.  The ReLU and the second layer (w1, b1) are applied in fp32
 * after the product.
 * ------------------------------------------------------------------------ */
typedef struct nglod_bf16_model {
    int32_t num_lods;
    int32_t base_lod;
    int32_t feature_dim;    /* 32 */
    int32_t hidden_dim;     /* 128 */
    const void  *grid[NGLOD_MAX_LODS];     /* bf16 channel-last [s][s][s][32], 16-byte aligned */
    const void  *w0_tile[NGLOD_MAX_LODS];  /* NGLOD_BF16_TILE_BYTES from nglod_bf16_pack_decoder */
    const float *b0[NGLOD_MAX_LODS];       /* [128]; informational (b0 is folded into w0_tile) */
    const float *w1[NGLOD_MAX_LODS];       /* [128] */
    const float *b1[NGLOD_MAX_LODS];       /* [1] */
    /* Optional pair volumes from nglod_bf16_build_pairs (32-byte aligned):
     * when set for every LOD a query reads, nglod_sdf_fwd_bf16 reads these
     * (one 128-byte line per vertex and its +x neighbour) instead of grid;
     * results are identical.  NULL: grid is read. */
    const void  *grid_pairs[NGLOD_MAX_LODS];
    /* Nonzero: grid[l] (and grid_pairs[l]) hold LOD-summed volumes from
     * nglod_build_summed_volume, and a query at lod L samples volume L alone
     * (one gather instead of L + 1).  0: per-LOD volumes, summed per query
     * as OctreeSDF.sdf does. */
    int32_t summed;
} nglod_bf16_model;

/* Pair volume of one bf16 volume grid [s][s][s][32]: pairs [s][s][s][2][32]
 * bf16, 128 bytes per vertex: four 32-byte units [v(z,y,x) channels 8c..8c+7
 * | v(z,y,min(x+1,s-1)) channels 8c..8c+7].  grid 16-byte aligned, pairs
 * 32-byte aligned, s in 2..1025. */
int nglod_bf16_build_pairs(const void *grid, int32_t s, void *pairs, nglod_stream_t stream);

/* LOD-summed volume `lod` of a float32 model: out[s][s][s][32] (s =
 * 2^(lod + base_lod) + 1, 16-byte aligned) of dtype NGLOD_F32 (float) or
 * NGLOD_BF16, vertex v = sum over LODs i <= lod of volume i's trilinear
 * sample (align_corners, border clamp) at v, computed in float64 and
 * rounded once.  Grid spacings halve from LOD to LOD, so each cell of LOD
 * `lod` lies inside one cell of every coarser grid and a trilinear sample
 * of out equals the running feature sum of OctreeSDF.sdf
 * (OctreeSDF.py:109-110) up to rounding.  Reads model->grid[0..lod] only.
 * bf16 volumes feed nglod_bf16_model with summed = 1; float volumes feed
 * nglod_sparse_build for nglod_sparse_model with summed = 1. */
int nglod_build_summed_volume(const nglod_dense_model *model, int32_t lod, int32_t dtype, void *out,
                              nglod_stream_t stream);

#define NGLOD_BF16_TILE_BYTES 12288

/* Host-only: lays out w0 [128][35] and b0 [128] (louts[i][0]) as the bf16 B
 * operand of the tensor-core tile (K-major, 8x8 core matrices, no swizzle),
 * NGLOD_BF16_TILE_BYTES bytes.  No CUDA calls. */
int nglod_bf16_pack_decoder(const float *w0_host, const float *b0_host, int32_t hidden_dim, int32_t in_dim,
                            void *tile_host);

/* OctreeSDF.sdf(x, lod) in the BF16 form: per-LOD bf16 trilinear gathers
 * summed in fp32, decoder on tcgen05 tensor cores (see above).
 * status: one device int32, set to nonzero if a bounded wait for the tensor
 * core gave up (the call zeroes it first). */
int nglod_sdf_fwd_bf16(const nglod_bf16_model *model, const float *x, int64_t n, int32_t lod, float *out,
                       int32_t *status, nglod_stream_t stream);

/* nglod_sdf_fwd_bf16 from host memory, pipelined as nglod_sdf_fwd_host. */
int nglod_sdf_fwd_bf16_host(const nglod_bf16_model *model, const float *x_host, int64_t n, int32_t lod,
                            float *out_host, int64_t chunk, void *scratch, int32_t *status, nglod_stream_t stream);

/* For tests of the error path: bounds the per-tile tensor-core waits of
 * later nglod_sdf_fwd_bf16 and tensor-core nglod_sdf_fwd / nglod_trace calls
 * (host setting, all devices) to `polls` polls of the mbarrier; 0 tests it
 * once without waiting (the float32 query, whose groups read a tile's
 * product back only after gathering their next tile, then also tests each
 * product right after issuing it), a negative value restores the default
 * (2^22 polls).  A wait that gives up sets the call's status, stops the
 * kernel after letting the issued product finish, and leaves the context
 * usable.  Not for production use. */
int nglod_debug_mma_wait_polls(int64_t polls);

/* Measurement helper, no reference counterpart: `blocks` blocks of 128
 * threads each read `loads` random whole 128-byte lines of buf[lines][128 B]
 * (32-byte aligned) with the point-query gather's 256-bit loads, four lanes
 * per line: blocks * 128 * loads * 32 bytes.  Timed around a buffer held in
 * L2, it gives the ceiling of the gather's corner reads.  sink: one device
 * uint32, written only to keep the loads. */
int nglod_measure_line_reads(const void *buf, int64_t lines, int32_t loads, int32_t blocks, uint32_t *sink,
                             nglod_stream_t stream);

/* Measurement helper, no reference counterpart: `blocks` blocks of 256
 * threads each run eight independent float32 FMA chains of `iters` steps,
 * blocks * 256 * 16 * iters FLOP.  Timed, it gives the float32 pipe's
 * throughput on this device.  sink: one device float, written only to keep
 * the chains. */
int nglod_measure_fma(int32_t iters, int32_t blocks, float *sink, nglod_stream_t stream);

/* Measurement helper, no reference counterpart: `blocks` blocks of 256
 * threads each read random whole 128-byte lines of a 32 KB shared-memory
 * buffer, eight lanes per line with one 16-byte load each, `loads` loads per
 * thread: blocks * 256 * 16 * loads bytes.  Timed, it gives the rate of the
 * SM's shared-memory / L1 data path for the float32 gather's line reads.
 * sink: one device uint32, written only to keep the loads. */
int nglod_measure_smem_reads(int32_t loads, int32_t blocks, uint32_t *sink, nglod_stream_t stream);

/* SphereTracer.forward in the BF16 form: the persistent tracer of
 * nglod_trace with every sdf evaluation (march points and normal taps) done
 * by the bf16 tile kernel above, 128 rays per block evaluated together.
 * Same outputs and march rules as nglod_trace, except that the ray
 * parameter t is accumulated as a compensated fp32 sum (TwoSum per step).
 * status: one device int32, nonzero if a bounded tensor-core wait gave up. */
int nglod_trace_bf16(const nglod_bf16_model *model, const nglod_trace_params *params, const float *ray_o,
                     const float *ray_d, int64_t n, float *x, float *t, uint8_t *hit, float *normal,
                     int64_t *work_counter, int32_t *status, nglod_stream_t stream);

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
 * (OctreeSDF.py:94-146); with all bits set, as sdf(x, return_lst=True).
 * relu_masks (optional, 16-byte aligned): relu_masks[l][n][(H+31)/32] gets
 * the decoder's ReLU mask (bit j of word j/32: hidden unit j was positive),
 * which nglod_sdf_bwd takes as the ReLU derivative, as autograd takes the
 * forward's saved activation.  With hidden_dim 128 and relu_masks given,
 * the decoders run on tcgen05 tensor cores: three TF32 products over
 * big / small splits of both operands (relative error about 2^-21), and
 * hidden units whose product lies within 1e-5 of zero evaluated again in
 * float32, so the ReLU decisions are the float32 path's.  That form writes
 * every feats row 0..L and reports a tensor-core wait that gives up through
 * nglod_train_status. */
int nglod_sdf_fwd_train(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                        float *preds, float *feats, uint32_t *relu_masks, nglod_stream_t stream);

/* Backward of nglod_sdf_fwd_train.  grad_preds[l][n] = dLoss/dpred_l for l in
 * lod_mask.  Adds the parameter gradients into `grads` and, when grad_x is
 * not NULL, dLoss/dx into grad_x[n][3].  dfeat_scratch[L+1][n][C] is caller-
 * provided scratch.  Replaces the autograd backward of OctreeSDF.sdf through
 * nn.Linear and F.grid_sample (border padding, align_corners) that
 * Trainer.step_geometry runs (sdf-net/lib/trainer.py:339).  With
 * hidden_dim 128 and the forward's relu_masks, the decoder part runs on
 * tcgen05 tensor cores (two products per 128-point tile, each as three
 * bf16 MMAs over hi / lo splits, fp32 accumulation: relative error about
 * 2^-16 per product, ReLU derivative from relu_masks); otherwise (relu_masks
 * NULL, or other widths) float32 tile reductions that recompute the hidden
 * layer in the forward's order.  Feature gradients are a trilinear
 * scatter-add (coarse volumes accumulated in shared memory, the rest with
 * vector atomics).  A tensor-core wait that gives up is reported by
 * nglod_train_status. */
int nglod_sdf_bwd(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                  const float *grad_preds, const float *feats, const uint32_t *relu_masks, float *dfeat_scratch,
                  const nglod_dense_grads *grads, float *grad_x, nglod_stream_t stream);

/* Reads and clears the training device status on the current device
 * (synchronous): *status_out = 1 if a bounded tensor-core wait of a
 * nglod_sdf_fwd_train, nglod_sdf_bwd or nglod_sdf_bwd_noalloc call since
 * the last read gave up (its outputs are incomplete), else 0. */
int nglod_train_status(int32_t *status_out);

/* nglod_sdf_bwd for callers that cannot allocate device memory (a plugin
 * whose GPU memory is owned by its host application, a process whose
 * allocator is locked after start-up): the same backward, but the per-point
 * scratch comes from a fixed array inside the library instead of a
 * caller-provided buffer, and the call allocates nothing.  No counterpart in
 * the reference.
 * Limit: (highest LOD in lod_mask + 1) * n * feature_dim floats must fit in
 * NGLOD_NOALLOC_SCRATCH_BYTES (16 MiB on every GPU that loads the library,
 * held until exit): n <= 26,214 with 5 LODs, 131,072 with one; larger n
 * returns NGLOD_ERR_CAPACITY.  The array's device address belongs to the
 * CUDA context: every call made outside stream capture looks it up
 * (cudaGetSymbolAddress) for the current context and caches it per context;
 * a call made while its stream is capturing uses the cache only.  So make
 * the first call in each context -- and again after cudaDeviceReset or after
 * creating a new context -- before any stream capture in it.  All calls
 * share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
#define NGLOD_NOALLOC_SCRATCH_BYTES (16u << 20)
int nglod_sdf_bwd_noalloc(const nglod_dense_model *model, const float *x, int64_t n, uint32_t lod_mask,
                          const float *grad_preds, const float *feats, const uint32_t *relu_masks,
                          const nglod_dense_grads *grads, float *grad_x, nglod_stream_t stream);

/* The loss of Trainer.step_geometry (sdf-net/lib/trainer.py:325-336) over
 * preds[rows][n] (rows = highest LOD + 1, as nglod_sdf_fwd_train writes them)
 * and gts[n]: *loss_out = sum over LODs l in lod_mask of
 * ((preds[l] - gts)^2).sum() / n to float64 accuracy (float-float partial
 * sums in float32 arithmetic, float64 across warps and blocks); and its
 * gradient grad_preds[l][q] = 2 (preds[l][q] - gts[q]) / n for l in the mask,
 * 0 for the other rows (the grad_preds of nglod_sdf_bwd).  One launch. */
int nglod_l2_loss(const float *preds, const float *gts, int64_t n, int32_t rows, uint32_t lod_mask,
                  double *loss_out, float *grad_preds, nglod_stream_t stream);

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

/* ------------------------------------------------------------------------
 * Structured point cloud (SPC) octree: build, decode, ray traversal.
 *
 * An octree of `level` levels is the sequence of child-occupancy bytes of
 * every occupied node of levels 0..level-1, level by level, each level in
 * Morton order (bit j of a node's byte = child j, j = 4*x + 2*y + z of the
 * child's offset).  Points are int16 [psize][4] (x, y, z, 0), all levels
 * concatenated (level 0 = the root).  pyramid is int32 [2][level+2]:
 * row 0 = points per level (then 0), row 1 = exclusive prefix sums
 * (row1[level+1] = psize).  Same formats as sol-renderer's SPC
 * (include/spc/spc/SPC.h:65-138, SPC.cu:148-238) and spc3d.SPC3D.
 * ------------------------------------------------------------------------ */

/* Octree from leaf voxels: pts[n][3] uint16 at `level` (duplicates allowed,
 * any order).  Writes octree bytes (capacity octree_cap), their count to
 * *osize, and pyramid[2][level+2].  scratch: at least
 * nglod_spc_build_scratch_bytes(level) bytes.  Bit-exact with
 * spc3d.SPC3D.points_to_nodes after Morton sorting (sdf-net/lib/spc3d.py:224-255).
 * Synchronises the stream once to return the sizes. */
int64_t nglod_spc_build_scratch_bytes(int32_t level);
int nglod_spc_build(const uint16_t *pts, int64_t n, int32_t level, uint8_t *octree, int64_t octree_cap,
                    int64_t *osize, int32_t *pyramid_host, void *scratch, nglod_stream_t stream);

/* SPC::SetGeometry (SPC.cu:148-238): octree bytes -> points[psize][4] int16
 * (capacity points_cap), exclusive prefix sums of child counts
 * prefix[osize+1] (prefix[k] = number of children of nodes before k; the
 * table the traversal addresses children with), and pyramid[2][level+2].
 * Synchronises the stream once to return the level sizes. */
int nglod_spc_decode(const uint8_t *octree, int64_t osize, int16_t *points, int64_t points_cap,
                     uint32_t *prefix, int32_t *pyramid_host, int32_t *level_out, nglod_stream_t stream);

/* spc_raytrace (include/spc/spc/spc_raytrace_cuda.cpp:141-199,
 * spc_raytrace_cuda_kernel.cu:194-265): level-by-level ray/voxel tests of
 * rays org/dir [n][3] against the octree down to target_level, children
 * expanded front to back.  Output: nuggets (ray index, level-local voxel
 * index) of every voxel at target_level the ray's line passes through, per
 * ray front to back, rays in order -- bit-exact with the reference.  All
 * levels run on the device with no host round trip.
 * nuggets_a/nuggets_b: two int32 [capacity][2] buffers; info: uint32
 * [max(capacity, 1024)], 8-byte aligned (chunk tickets and scan states);
 * partials: uint32 [capacity/1024 + 2] (not used by this entry point; kept
 * for the signature); ctrl: int64 [NGLOD_SPC_CTRL_WORDS] device.
 * One launch per level: each 1024-nugget chunk finds its output offset by
 * a bounded look-back over the preceding chunks (NGLOD_ERR_CUDA if a wait
 * gave up).
 * On return (the call synchronises once) *count = number of nuggets and
 * *result_buffer = 0 (nuggets_a) or 1 (nuggets_b) holds them.  More than
 * `capacity` nuggets at any level: NGLOD_ERR_CAPACITY (the reference
 * truncated silently).  capacity < 2^29, so that a level's count (at most
 * eight children per nugget) stays below 2^32. */
/* Exclusive prefix sums of child counts over all octree bytes:
 * prefix[k] = sum of popcount(octree[i]) for i < k, k in [0, osize]; the
 * table the reference recomputes on every spc_raytrace call with CUB
 * (spc_raytrace_cuda_kernel.cu:226-227).  partials: uint32
 * [osize/1024 + 2]; ctrl: int64 [2].  Asynchronous. */
int nglod_spc_prefix(const uint8_t *octree, int64_t osize, uint32_t *prefix, uint32_t *partials, int64_t *ctrl,
                     nglod_stream_t stream);

#define NGLOD_SPC_CTRL_WORDS 20
int nglod_spc_raytrace(const uint8_t *octree, const int16_t *points, const uint32_t *prefix,
                       const int32_t *pyramid_host, int32_t level, int32_t target_level,
                       const float *org, const float *dir, int64_t n_rays,
                       int32_t *nuggets_a, int32_t *nuggets_b, int64_t capacity, uint32_t *info,
                       uint32_t *partials, int64_t *ctrl, int64_t *count, int32_t *result_buffer,
                       nglod_stream_t stream);

/* d_MarkUniqueRays (sol-renderer/sdfRenderer.cu:108-120): info[i] = 1 where
 * nugget i is its ray's first, else 0. */
int nglod_spc_mark_first(const int32_t *nuggets, int64_t n, int32_t *info, nglod_stream_t stream);

/* Octree from a field (the purpose of voxel_sparsify,
 * sdf-net/lib/renderutils.py:56-73, as SOL_NGLOD.py:50 uses it):
 * _voxel_centres writes the centres float32 [count][3] of voxels
 * [start, start + count) of the 2^level grid over [-1, 1]^3, linear index
 * (x * res + y) * res + z; after the caller evaluates the field there,
 * _select_band appends the uint16 (x, y, z) of the voxels with |value| <= band
 * to voxels[base ..], fails with NGLOD_ERR_CAPACITY past `capacity`, and
 * returns their number in *selected (host; the call waits for it).
 * partials: n/1024 + 2 uint32; ctrl: 3 int64.  The voxels feed
 * nglod_spc_build.  No reference counterpart for the band rule itself. */
int nglod_voxel_centres(int32_t level, int64_t start, int64_t count, float *out, nglod_stream_t stream);
int nglod_select_band(const float *values, int64_t n, float band, int32_t level, int64_t start, uint16_t *voxels,
                      int64_t base, int64_t capacity, uint32_t *partials, int64_t *ctrl, int64_t *selected,
                      nglod_stream_t stream);

/* spc_generate_primary_rays (spc_raytrace_cuda.cpp:65-121, kernel
 * spc_raytrace_cuda_kernel.cu:271-287): pinhole rays of a width x height
 * image from the 4x4 inverse view-projection matrix inv_wvp (row-major,
 * row-vector convention); directions are not normalised, as in the
 * reference. */
int nglod_spc_generate_rays(const float *inv_wvp_host, int32_t width, int32_t height, float *org, float *dir,
                            nglod_stream_t stream);

/* ------------------------------------------------------------------------
 * Sparse SDF on an SPC octree (sol-renderer's SDF class, SDF.h:44-97).
 *
 * LOD i lives on octree level i + 2.  The features of the unique corners of
 * the occupied voxels of every level are stored once (all levels
 * concatenated, each level's corners in lexicographic (x, y, z) order, as
 * SOL_NGLOD exports them: sdf-net/lib/models/SOL_NGLOD.py:68-75).  For every
 * octree point of level >= 2, corner_idx[p][8] holds the global corner index
 * of its 8 corners (corner j = (x + (j>>2&1), y + (j>>1&1), z + (j&1))) and
 * parent[p] the global point index of its parent (-1 at level 2): the
 * reference's Trinket {v[8], parent} (solr/util_structs.cuh:33-37).
 * ------------------------------------------------------------------------ */
typedef struct nglod_sparse_model {
    int32_t num_lods;        /* decoders; octree levels 2 .. num_lods + 1 */
    int32_t feature_dim;     /* 32 */
    int32_t hidden_dim;      /* <= 256, even */
    int32_t feat_dtype;      /* NGLOD_F32 or NGLOD_BF16 corner features */
    const void    *corner_feats;  /* [ncorners][feature_dim], 16-byte aligned */
    const int32_t *corner_idx;    /* [psize][8], 16-byte aligned */
    const int32_t *parent;        /* [psize] */
    const int16_t *points;        /* [psize][4] */
    int64_t level_start[16];      /* global index of each octree level's first point */
    const float *w0[NGLOD_MAX_LODS];
    const float *b0[NGLOD_MAX_LODS];
    const float *w1[NGLOD_MAX_LODS];
    const float *b1[NGLOD_MAX_LODS];
    /* optional: NGLOD_BF16_TILE_BYTES decoder tiles (nglod_bf16_pack_decoder)
     * for nglod_sparse_trace_tc; unused by the other calls */
    const void *w0_tile[NGLOD_MAX_LODS];
    /* optional, per lod: corner_chain[lod][v][k][8] = corner_idx of the
     * level-(lod+2-k) ancestor of voxel v of level lod+2 (k = 0..lod), from
     * nglod_sparse_build_chain, 16-byte aligned.  When set,
     * nglod_sparse_trace_tc reads a voxel's corners of every level from its
     * own row instead of walking `parent` (identical results). */
    const int32_t *corner_chain[NGLOD_MAX_LODS];
    /* Nonzero: corner_feats come from LOD-summed volumes
     * (nglod_build_summed_volume, then nglod_sparse_build), and every query
     * at lod L samples the corners of its level-(L+2) voxel alone instead of
     * adding its ancestors' samples (equal up to rounding: each ancestor
     * contains the point). */
    int32_t summed;
} nglod_sparse_model;

/* SDF::initTrinkets + the corner export of SOL_NGLOD (SDF.cu:141-216,
 * SOL_NGLOD.py:68-75): from a dense model whose LOD i volume has
 * 2^(i+2)+1 vertices per side and an octree with at least num_lods + 1
 * levels, writes corner features (corner_cap rows, dtype feat_dtype),
 * corner_idx, parent, and corner_counts_host[num_lods] (corners per LOD).
 * scratch: nglod_sparse_build_scratch_bytes(level) bytes.  Replaces the
 * reference's O(points x corners) search (solr/sdf/index_trinket.cuh:31-98)
 * with dense index grids.  Synchronises once. */
int64_t nglod_sparse_build_scratch_bytes(int32_t level);
int nglod_sparse_build(const nglod_dense_model *dense, const int16_t *points, const int32_t *pyramid_host,
                       int32_t level, int32_t feat_dtype, void *corner_feats, int64_t corner_cap,
                       int32_t *corner_idx, int32_t *parent, int64_t *corner_counts_host, void *scratch,
                       nglod_stream_t stream);

/* SDF::forward(x, lod) -- declared in SDF.h:52-54 but never defined in the
 * reference: the sparse SDF at points x[n][3].  Each point's voxel at octree
 * level lod+2 is found by descending the octree (spc3d.SPC3D.Identify,
 * sdf-net/lib/spc3d.py:309-338); points outside every occupied voxel get
 * NaN.  octree/prefix as from nglod_spc_decode. */
int nglod_sparse_query(const nglod_sparse_model *model, const uint8_t *octree, const uint32_t *prefix, int32_t lod,
                       const float *x, int64_t n, float *out, nglod_stream_t stream);

/* SDF::sphereTrace (SDF.cu:297-472, kernels solr/sdf/sparse_grid_sample.cuh,
 * solr/sdf/step.cuh, solr/gfx/ray_aabb.cuh, solr/common/normalize.cuh) in one
 * persistent launch.  nuggets[m][2] from nglod_spc_raytrace at level lod+2;
 * rays without nuggets are left untouched by the march (t = 0, x = ray_o,
 * hit = 0, normal = (1,1,1)).  Per ray: voxel walk from ray_o, then up to
 * num_steps sparse evaluations (t += d; hit = |d| < 3e-4 or
 * |d + dprev|/2 < 1.5e-3; stop at t >= 5 or leaving the voxels, t = 100),
 * normals of hit rays by central differences (1e-3) inside the last voxel.
 * ray_first: int32 [n] scratch; work_counter: one int64. */
int nglod_sparse_trace(const nglod_sparse_model *model, int32_t lod, int32_t num_steps, const float *ray_o,
                       const float *ray_d, int64_t n, const int32_t *nuggets, int64_t n_nuggets,
                       int32_t *ray_first, float *x, float *t, uint8_t *hit, float *normal, int64_t *work_counter,
                       nglod_stream_t stream);

/* Fills chain [count][lod+1][8] int32 (count = level_start[lod+3] -
 * level_start[lod+2] voxels of level lod+2) for model->corner_chain[lod]:
 * row v, block k = corner_idx of the voxel reached from voxel v by k parent
 * steps.  Needs corner_idx and parent of the model. */
int nglod_sparse_build_chain(const nglod_sparse_model *model, int32_t lod, int64_t count, int32_t *chain,
                             nglod_stream_t stream);

/* nglod_sparse_trace with bf16 corner features and the BF16 decoder of
 * nglod_sdf_fwd_bf16: every sdf evaluation of 128 rays is one tcgen05 tile
 * product (model->w0_tile[lod] required; feature_dim 32, hidden_dim 128).
 * Same march, walk and normal rules as nglod_sparse_trace.  status: one
 * device int32, nonzero if a bounded tensor-core wait gave up.  No reference
 * counterpart (the reference decodes with cuBLAS in float32, SDF.cu:420-421). */
int nglod_sparse_trace_tc(const nglod_sparse_model *model, int32_t lod, int32_t num_steps, const float *ray_o,
                          const float *ray_d, int64_t n, const int32_t *nuggets, int64_t n_nuggets,
                          int32_t *ray_first, float *x, float *t, uint8_t *hit, float *normal, int64_t *work_counter,
                          int32_t *status, nglod_stream_t stream);

/* ------------------------------------------------------------------------
 * Mesh data path: signed distance of points to a triangle mesh
 * (compute_sdf -> mesh2sdf.mesh2sdf_gpu, sdf-net/lib/torchgp/compute_sdf.py:
 * 26-40; the algorithm of sdf-net/lib/extensions/mesh2sdf_cuda/
 * mesh2sdf_kernel.cu:307-617: minimum point-triangle distance, negative when
 * each of 13 fixed lines through the point crosses the mesh on both sides).
 * ------------------------------------------------------------------------ */

/* Floats per triangle record (nglod_mesh_prepare's output stride). */
int64_t nglod_mesh_record_floats(void);

/* triangles float32 [m][3][3] (vertices of each face) -> records
 * [m][nglod_mesh_record_floats()], 16-byte aligned. */
int nglod_mesh_prepare(const float *triangles, int64_t m, float *records, nglod_stream_t stream);

/* out[n] = signed distance of points [n][3] to the mesh of m records. */
int nglod_mesh_sdf(const float *records, int64_t m, const float *points, int64_t n, float *out,
                   nglod_stream_t stream);

/* ------------------------------------------------------------------------
 * Shading passes on a traced render buffer (Renderer.render / shade_tensor,
 * sdf-net/lib/renderer.py:118-223; geoutils.py:237-276).  Buffers are the
 * tracer's: x [n][3], t [n], hit [n], normal [n][3]; images are [W][H]
 * with ray i = w * H + h (nglod_camera_rays' order).
 * ------------------------------------------------------------------------ */

/* Lowest y of the hit points, as an order-preserving uint32 key in *out_key
 * (device): key = bits | 0x80000000 for y >= 0, ~bits for y < 0;
 * 0xFFFFFFFF when nothing was hit.  (renderer.py:76-86 takes the ground
 * height from the lowest surface sample.) */
int nglod_shade_min_hit_y(const float *x, const uint8_t *hit, int64_t n, uint32_t *out_key, nglod_stream_t stream);

/* Ground plane y = min_y (renderer.py:131-150): where the plane is nearer than
 * the surface (0 < t_plane < min(500, t)), x / t / normal become the plane's
 * and hit is cleared; plane_hit [n] marks those rays. */
int nglod_shade_ground(const float *ray_o, const float *ray_d, int64_t n, float min_y, float *x, float *t,
                       uint8_t *hit, float *normal, uint8_t *plane_hit, nglod_stream_t stream);

/* Shadow rays (renderer.py:152-161): origin x + 0.1 normal, direction
 * normalize(noise + light - origin) with the caller's N(0, 0.01^2) noise
 * [n][3]; light_host float[3] (the reference's (-1.5, 4.5, -1.5));
 * light_hit = direction . normal > 0.  Trace them with nglod_trace(_bf16). */
int nglod_shade_shadow_rays(const float *x, const float *normal, const float *noise, int64_t n,
                            const float *light_host, float *shadow_o, float *shadow_d, uint8_t *light_hit,
                            nglod_stream_t stream);

/* Ambient occlusion (renderer.py:184-208) in three calls: _ao_select writes
 * the indices of the shaded rays (hit, or plane_hit when given; plane_hit may
 * be NULL) to idx [n] and their number to *count (host; the call waits for
 * it; partials [n/1024 + 2], ctrl [2] int64 scratch); _ao_taps writes the 40
 * tap points x + normal * d_i of each selected ray to taps [count*40][3],
 * d_i = 0.025 ((i+1)/41)^1.6; the caller evaluates the sdf at the taps (any
 * nglod_sdf_fwd* call) into r [count*40]; _ao_reduce writes ao [n] =
 * clamp(1 - sum_i 3.5 relu(d_i - r_i - 0.0015), 0.1, 1)^2 (1 for rays not
 * selected; a plane ray's r_i is min(r_i, d_i)). */
int nglod_shade_ao_select(const uint8_t *hit, const uint8_t *plane_hit, int64_t n, int32_t *idx, uint32_t *partials,
                          int64_t *ctrl, int64_t *count, nglod_stream_t stream);
int nglod_shade_ao_taps(const float *x, const float *normal, const int32_t *idx, int64_t count, float *taps,
                        nglod_stream_t stream);
int nglod_shade_ao_reduce(const float *r, const int32_t *idx, int64_t count, const uint8_t *plane_hit, int64_t n,
                          float *ao, nglod_stream_t stream);

/* Matcap colour (renderer.py:262-279 with geoutils.spherical_envmap and a
 * bilinear matcap_sampler): rgb [n][3] in [0, 1] for hit rays, 1 elsewhere.
 * view = ray directions; texture float32 [tex_w][tex_h][3] in 0..255 (the
 * reference's image transposed to (width, height)). */
int nglod_shade_matcap(const float *view, const float *normal, const uint8_t *hit, int64_t n, const float *texture,
                       int32_t tex_w, int32_t tex_h, float *rgb, nglod_stream_t stream);

/* Shadow map (renderer.py:283-286): shadow [rows*cols] = shadow_hit &
 * light_hit; map = gaussian_filter(clamp(1 - shadow + 0.9, 0, 1), sigma)
 * (scipy.ndimage, mode 'reflect', truncate 4) over the [rows][cols] image;
 * scratch: rows*cols floats. */
int nglod_shade_shadow_map(const uint8_t *shadow_hit, const uint8_t *light_hit, int32_t rows, int32_t cols,
                           float sigma, float *map, float *scratch, uint8_t *shadow, nglod_stream_t stream);

/* rgb (if given) *= shadow_map (if given) * ao (if given); relative_depth
 * (if given) = clamp(t, 0, far_clip) / far_clip (renderer.py:167). */
int nglod_shade_compose(float *rgb, int64_t n, const float *shadow_map, const float *ao, const float *t,
                        float far_clip, float *relative_depth, nglod_stream_t stream);

/* ------------------------------------------------------------------------
 * Serving: a continuous-batching request server over resident models.
 *
 * No reference counterpart: the reference renders one frame at a time in
 * its viewer loop (sol-renderer/sdfRenderer.cpp:217-242) and answers point
 * queries only through OctreeSDF.sdf.  The server keeps models resident and
 * takes render and point-query requests as they arrive.  A request is
 * admitted, in arrival order, as soon as (a) its device state fits in the
 * server's pool of hbm_budget_bytes (first fit, 256-byte aligned regions)
 * and (b) one of num_slots slots is free; each slot owns a CUDA stream, so
 * admitted requests of different models, sizes and LODs run on the GPU at
 * the same time.  Completion is detected by polling CUDA events (never a
 * blocking device wait).  Every kernel computes each ray / point on its own,
 * so a result is bitwise the same alone and in any mix.
 *
 * Ownership: the server owns its pool (allocated once at start), its streams
 * and events.  Results live in the pool until nglod_serve_release.  Models
 * and query points are the caller's device memory, borrowed: models until
 * nglod_serve_destroy, points until their request has completed.
 * Thread safety: every call locks the server; calls from several threads
 * are serialised.
 * ------------------------------------------------------------------------ */
typedef struct nglod_server nglod_server; /* opaque */

#define NGLOD_SERVE_RENDER 1
#define NGLOD_SERVE_QUERY  2

typedef struct nglod_serve_config {
    int64_t hbm_budget_bytes; /* pool size: device state of requests on the GPU plus unreleased results */
    int32_t num_slots;        /* requests on the GPU at once, one CUDA stream each, 1..64 */
    int32_t reserved;
} nglod_serve_config;

typedef struct nglod_serve_request {
    int32_t kind;                /* NGLOD_SERVE_RENDER or NGLOD_SERVE_QUERY */
    int32_t model;               /* id from nglod_serve_add_model_* */
    int32_t lod;                 /* LOD of every sdf evaluation; <0: finest */
    int32_t width, height;       /* render: image size; rays as nglod_camera_rays */
    float eye[3], at[3], up[3];  /* render: camera */
    float fov_deg;               /* render */
    nglod_trace_params trace;    /* render: march parameters (its lod field is ignored) */
    const float *points;         /* query: device [n][3] float32 */
    int64_t n;                   /* query: number of points */
    int32_t has_ready_stream;    /* 1: the request's work first waits for the work queued on ready_stream */
    int32_t reserved;            /*    at submit time (the stream that wrote `points`) */
    nglod_stream_t ready_stream;
} nglod_serve_request;

typedef struct nglod_serve_result {
    int64_t ticket;
    int32_t kind;
    int32_t status;         /* NGLOD_OK, or the error code of the request's launch or run */
    double t_submit;        /* host monotonic clock (CLOCK_MONOTONIC), seconds */
    double t_admit;
    double t_done;          /* when a poll first saw the request finished */
    int64_t units;          /* rays (render) or points (query) */
    float *x;               /* render: [units][3] hit points (device, in the pool) */
    float *t;               /* render: [units] depth */
    uint8_t *hit;           /* render: [units] */
    float *normal;          /* render: [units][3] */
    float *sdf;             /* query: [units] distances */
} nglod_serve_result;

typedef struct nglod_serve_info {
    int64_t budget_bytes, used_bytes, peak_used_bytes;
    int32_t num_slots, pending, running, unpolled, held, max_concurrent;
    int64_t submitted, completed;
} nglod_serve_info;

/* Device bytes a request takes from the pool (0 for an invalid request). */
int64_t nglod_serve_request_bytes(const nglod_serve_request *request);

/* Creates a server on the current CUDA device. */
int nglod_serve_start(const nglod_serve_config *config, nglod_server **server);

/* Registers a resident model (the descriptor is copied; the memory it points
 * to stays the caller's).  *model_id: its index, from 0. */
int nglod_serve_add_model_f32(nglod_server *server, const nglod_dense_model *model, int32_t *model_id);
int nglod_serve_add_model_bf16(nglod_server *server, const nglod_bf16_model *model, int32_t *model_id);

/* Queues a request.  t_arrival: its arrival time on the host monotonic clock
 * (seconds; < 0: now), the start of its latency.  Admits whatever fits.
 * NGLOD_ERR_CAPACITY if the request alone needs more than the whole pool. */
int nglod_serve_submit(nglod_server *server, const nglod_serve_request *request, double t_arrival,
                       int64_t *ticket);

/* Retires finished requests, admits waiting ones, and returns up to
 * max_results finished requests (each once, in completion order). */
int nglod_serve_poll(nglod_server *server, nglod_serve_result *results, int32_t max_results, int32_t *count);

/* Returns a polled request's region to the pool.  has_stream = 1: the region
 * is reused only after the work queued on `stream` now (e.g. copies of the
 * results) has finished. */
int nglod_serve_release(nglod_server *server, int64_t ticket, int32_t has_stream, nglod_stream_t stream);

int nglod_serve_get_info(nglod_server *server, nglod_serve_info *info);

/* Bounded shutdown: drops the waiting requests, stops admitting, and polls
 * the running ones for up to timeout_s seconds.  Finished requests stay
 * pollable.  *unfinished: requests still on the GPU; *dropped: requests
 * that never started. */
int nglod_serve_stop(nglod_server *server, double timeout_s, int32_t *unfinished, int32_t *dropped);

/* Waits for the server's streams, frees the pool, streams and events. */
int nglod_serve_destroy(nglod_server *server);

/* A server over caller-supplied launch / completion callbacks instead of
 * CUDA (embedding in another runtime; scheduling tests on hosts without a
 * GPU).  The pool is not allocated: regions are byte offsets, and result
 * pointers are those offsets.  Callbacks run with the server locked and
 * must not call the server. */
typedef struct nglod_serve_executor {
    void *ctx;
    /* starts `request` in `slot` in pool region [region, region + bytes); 0 or an error code */
    int32_t (*launch)(void *ctx, int64_t ticket, int32_t slot, const nglod_serve_request *request, int64_t region,
                      int64_t bytes);
    /* 1: the request in `slot` has finished; 0: still running; < 0: it failed with that code */
    int32_t (*query)(void *ctx, int64_t ticket, int32_t slot);
} nglod_serve_executor;
int nglod_serve_start_custom(const nglod_serve_config *config, const nglod_serve_executor *executor,
                             nglod_server **server);

#ifdef __cplusplus
}
#endif

#endif /* NGLOD_GB300_H */
