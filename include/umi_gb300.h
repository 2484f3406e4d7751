/* umi_gb300: C ABI of the GB300 (sm_103a) implementation of the UMI operator.
 *
 * Everything here is plain C: raw device pointers, sizes, and a CUDA stream
 * passed as `void*` (a cudaStream_t; NULL = the legacy default stream).  All
 * entry points are asynchronous on that stream, never allocate device memory
 * unless stated, keep no mutable global state beyond what is stated (the
 * built-in scratch of umi_iimg_u8_i32_noalloc, the per-thread second stream
 * of the motion-estimation pipelines), and report failures by status code
 * (the reference aborts or ignores CUDA errors instead).
 *
 * The reference exposes one templated entry point, UMI::Execute
 * (src/UMI_gpu.h:409-623).  Its two halves map onto this library as:
 *   - validation + tiling (src/UMI.cpp:39-76, src/UMI_gpu.h:423-609)
 *       -> umi_plan_build(), consumed by the header-only generic kernel in
 *          include/umi/UMI_gpu.h (user functors are device code and must be
 *          compiled in the caller's translation unit);
 *   - the example applications (main/<app>.cu) -> the specialised
 *     umi_<op>_<dtype> kernels below, each citing the application it
 *     replaces.
 */
#ifndef UMI_GB300_H
#define UMI_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* status                                                              */
/* ------------------------------------------------------------------ */
typedef enum umi_status {
	UMI_OK = 0,
	UMI_ERR_INVALID_DESC = 1, /* descriptor rejected (reference: abort() at src/UMI.cpp:60,64) */
	UMI_ERR_INVALID_ARG = 2,  /* null pointer, negative size, misaligned buffer */
	UMI_ERR_UNSUPPORTED = 3,  /* valid request outside what this build implements */
	UMI_ERR_CUDA = 4,         /* a CUDA runtime call failed (reference: ignored) */
	UMI_ERR_NO_MEMORY = 5,    /* workspace too small */
	UMI_ERR_TIMEOUT = 6       /* a bounded device-side wait gave up */
} umi_status;

/* Human-readable name of a status code. */
const char* umi_status_string(int status);
/* Detail of the last failure on the calling host thread ("" if none). */
const char* umi_last_error_string(void);
/* Library version, major*10000 + minor*100 + patch. */
int umi_version(void);

/* ------------------------------------------------------------------ */
/* generic operator: descriptor validation and tiling                  */
/* ------------------------------------------------------------------ */
#define UMI_DIM 4
#define UMI_MAX_PTR 4
#define UMI_MAX_MEMS 16

/* POD mirrors of the descriptor types of src/UMI.h:77-93. */
typedef struct { int32_t total_size, block_size, warp_size, warp_shuf; } umi_pdim;
typedef struct { int32_t total_size, block_size; } umi_adim;
typedef struct { int32_t physical_dim_id, ofs, stride; } umi_vdim;
typedef struct { int32_t size, mode; } umi_phydim; /* mode 0 = PAD, 1 = WRAP (clamp) */

/* One memory (input or output) of a call.  stage: 0 Pre, 1 Loop, 2 Post. */
typedef struct {
	umi_vdim p_view[UMI_DIM];
	umi_vdim a_view[UMI_DIM];
	umi_phydim phys[UMI_DIM];
	int32_t stage;
	int32_t n_ptr;
} umi_mem_desc;

/* A whole call: src/UMI_gpu.h:416-422 without the pointers.  Memories are
 * ordered like the reference: inputs (Pre, Loop, Post), then outputs
 * (Pre, Loop, Post).  expand is the 16-bit Expand word (E0 = nibble 3). */
typedef struct {
	umi_pdim p[UMI_DIM];
	umi_adim a[UMI_DIM];
	uint32_t expand;
	int32_t n_in, n_out;
	umi_mem_desc mem[UMI_MAX_MEMS];
} umi_desc;

/* Per-memory closed-form address map: physical coordinate k of the element
 * read/written for point p and accumulation index a is
 *   base[k] + sum_d pcoef[k][d]*p[d] + sum_d acoef[k][d]*a[d];
 * inputs clamp each coordinate to [0, size[k]-1] (pad_mask bit k: the value
 * becomes the padding value instead), outputs do not clamp.  The linear
 * element index is sum_k coord[k]*rowstride[k]. */
typedef struct {
	int32_t base[UMI_DIM];
	int32_t pcoef[UMI_DIM][UMI_DIM];
	int32_t acoef[UMI_DIM][UMI_DIM];
	int32_t size[UMI_DIM];
	int64_t rowstride[UMI_DIM];
	int32_t pad_mask;
	int32_t stage;
	int32_t n_ptr;
	int32_t is_output;
} umi_mem_plan;

/* Launch geometry of one call.  Tiling never changes results (only the
 * accumulation order is fixed: blocked row-major over A). */
typedef struct {
	int32_t ptotal[UMI_DIM];
	int32_t block[UMI_DIM];   /* threads per CTA along each P dim */
	int32_t expand[UMI_DIM];  /* points per thread along each P dim */
	int32_t grid[UMI_DIM];    /* CTAs along each P dim */
	int64_t n_cta;
	int32_t n_threads;
	int32_t atotal[UMI_DIM];
	int32_t ablock[UMI_DIM];
	int32_t agrid[UMI_DIM];
	int32_t n_ablock;         /* product of agrid (0 when A is empty) */
	int32_t ablock_size;      /* product of ablock */
	int32_t n_in, n_out;
	umi_mem_plan mem[UMI_MAX_MEMS];
} umi_plan;

/* Validate `desc` (same rules as src/UMI.cpp:39-66: the product of the
 * warp sizes is 32, every warp_shuf a power of two (0 read as 1), every
 * block_size divisible by warp_size*warp_shuf; plus: at most 1024 threads,
 * positive blocks, PtrNum nibbles <= 4, <= 16 memories) and fill `plan`.
 * Reference: PDims_packed / ADims_packed ctors + the table builders of
 * Execute (src/UMI.cpp:39-226, src/UMI_gpu.h:423-609), which abort instead of
 * returning UMI_ERR_INVALID_DESC. */
umi_status umi_plan_build(const umi_desc* desc, umi_plan* plan);

/* The same validation into a plan allocated by the library (host memory,
 * released by umi_plan_destroy).  Reference: the descriptor half of
 * Execute, src/UMI_gpu.h:423-609. */
umi_status umi_plan_create(const umi_desc* desc, umi_plan** plan);
void umi_plan_destroy(umi_plan* plan);

/* Strategies built into umi_launch: the functors of the reference's example
 * applications, same arithmetic, element type and constants. */
typedef enum umi_strategy {
	UMI_STRATEGY_NEIGHBOUR_SUM_I32 = 0,  /* main/filter3x3.cu:10-17: Pre t = init; Loop(1 in) t += x; Post out = t * mul; constants {int init, mul} */
	UMI_STRATEGY_WEIGHTED_SUM_I32 = 1,   /* main/wfilter3x3.cu:8-15: Pre t = init; Loop(2 in) t += x * w; Post out = t; constants {int init} */
	UMI_STRATEGY_RANGE_WEIGHTED_F32 = 2, /* main/bilateral.cu:9-24: Pre(1 in) centre; Loop(3 in) w = expf((x-centre)^2 * norm) * ws_y * ws_x; Post out = sum(w x) / sum(w); constants {float norm} */
	UMI_STRATEGY_ABS_DIFF_SUM_I32 = 3,   /* main/cost_volume.cu:8-15 and main/full_me.cu: Loop(2 in) s += |a - b|; Post out = s */
	UMI_STRATEGY_RUNNING_SUM_I32 = 4,    /* main/iimg.cu:11-18: Loop(1 in, 1 out) out = t += x */
	UMI_STRATEGY_DOT_I32 = 5,            /* main/gemm.cu:8-15 and main/fprop.cu: Loop(2 in) t += a * b; Post out = t */
	UMI_STRATEGY_DOT_F32 = 6,            /* the same on float */
	/* window operators of the same family (no reference example) */
	UMI_STRATEGY_CENSUS_I32 = 7,         /* Pre(1 in) centre; Loop(1 in) bits = bits << 1 | (x < centre); Post out = bits (last 32) */
	UMI_STRATEGY_WEIGHTED_SUM_F32 = 8,   /* Pre t = init; Loop(2 in) t = fma(x, w, t); Post out = t; constants {float init} */
	UMI_STRATEGY_MAX_I32 = 9,            /* Pre t = init; Loop(1 in) t = max(t, x); Post out = t; constants {int init} */
	UMI_STRATEGY_MIN_I32 = 10            /* Pre t = init; Loop(1 in) t = min(t, x); Post out = t; constants {int init} */
} umi_strategy;

/* Generic operator through the C ABI: runs `strategy` over the plan's P x A
 * space (the semantics of Execute, src/UMI_gpu.h:189-358: Pre, Loop over A
 * in blocked row-major order, Post, per-dimension clamp / PAD).  in[i] and
 * out[i] are the device pointers of the plan's inputs and outputs (one per
 * memory); pad (may be NULL = all zero) holds one 4-byte padding value per
 * input (UnrolledI::padding); user_const / uc_bytes the strategy's
 * constants.  The memories' count and stages must be the strategy's. */
umi_status umi_launch(const umi_plan* plan, int32_t strategy, const void* const* in, const void* pad,
                      void* const* out, const void* user_const, size_t uc_bytes, void* stream);

/* ------------------------------------------------------------------ */
/* specialised kernels                                                 */
/* ------------------------------------------------------------------ */

/* 3x3 weighted filter, float32, (h, w) row-major, out-of-image pixels read
 * as `pad`.  out[y,x] = sum_{dy,dx} w9[3*(dy+1)+(dx+1)] * in[y+dy, x+dx].
 * w9 is a HOST array of 9 floats (copied into the launch).  in/out must not
 * alias.  Replaces main/filter3x3.cu:37-58 and main/wfilter3x3.cu:39-69
 * (their Execute calls) for float images. */
umi_status umi_filter3x3_f32(const float* in, float* out, int32_t h, int32_t w, const float* w9, float pad,
                             void* stream);
/* The same filter with zero padding (PAD 0) through TMA-staged halo tiles:
 * one tensor-map box per 128 x 16 tile (the map's zero fill is the padding),
 * double-buffered in shared memory, TMA tile stores.  16-byte aligned in/out
 * and w % 4 == 0 (else UMI_ERR_UNSUPPORTED).  The staged form of the
 * reference's FillShm halo tile (src/UMI_gpu.h:33-83); measured slower than
 * umi_filter3x3_f32 on GB300 (which already reads each input once from HBM),
 * so it is not the default.  Same FMA order: results equal umi_filter3x3_f32
 * with pad 0 bit for bit. */
umi_status umi_filter3x3_f32_tma(const float* in, float* out, int32_t h, int32_t w, const float* w9, void* stream);

/* Integral image, uint8 -> int32: out[y,x] = sum_{y'<=y, x'<=x} in[y',x'].
 * Replaces the two Execute calls of main/iimg.cu:37-82 (row prefix through a
 * Loop output, transposed, twice) with two launches: column sums per group
 * of 128 rows, then one output pass.  Needs a device workspace of
 * umi_iimg_u8_i32_workspace_bytes(h, w) bytes (16-byte aligned; about
 * 0.27 byte per pixel; its content need not be initialised).  Frames with
 * h*w*255 >= 2^31 are rejected (UMI_ERR_UNSUPPORTED: sums could overflow
 * int32). */
size_t umi_iimg_u8_i32_workspace_bytes(int32_t h, int32_t w);
umi_status umi_iimg_u8_i32(const uint8_t* in, int32_t* out, int32_t h, int32_t w, void* workspace,
                           size_t workspace_bytes, void* stream);

/* The same integral image for callers that cannot allocate device memory
 * (no allocator to take a workspace from, or a context where cudaMalloc is
 * not allowed).  No counterpart in the reference.  The tile sums go to a
 * scratch array built into the library, UMI_IIMG_NOALLOC_SCRATCH_BYTES
 * (1 MiB) per GPU, held until the process exits; frames whose tile sums
 * (int32 per row per 256-column tile, per column per 64-row tile and per
 * tile, each array rounded up to 256 bytes) exceed it are rejected with
 * UMI_ERR_NO_MEMORY; at most 4096 rows.  The int32 limit of
 * umi_iimg_u8_i32 applies too (h*w*255 < 2^31: about 8.42 Mpx, so 3840x2160
 * is served and 4096x2160 is refused with UMI_ERR_UNSUPPORTED).  The first
 * call in a CUDA context looks up the scratch address (cudaGetSymbolAddress)
 * with that context current and caches it per context: make it before any
 * stream capture.  All calls share the scratch: calls that overlap on the
 * GPU race and must be serialised by the caller.  Allocates nothing. */
#define UMI_IIMG_NOALLOC_SCRATCH_BYTES (1u << 20)
umi_status umi_iimg_u8_i32_noalloc(const uint8_t* in, int32_t* out, int32_t h, int32_t w, void* stream);
/* Drops the cached scratch addresses of umi_iimg_u8_i32_noalloc: call it
 * after a context it served was destroyed (cudaDeviceReset), before the next
 * call.  No counterpart in the reference. */
void umi_iimg_noalloc_forget(void);

/* Full-search block motion estimation with fused argmin, uint8 frames.
 * For every b x b block of `cur` (blocks truncated at the frame edge:
 * h/b x w/b, as main/full_me.cu:35), searches displacements (dy, dx) in
 * [cy-r, cy+r] x [cx-r, cx+r] of `ref`, where (cy, cx) is the block's search
 * centre (0,0 when `centers` is NULL, else centers[2*blk], centers[2*blk+1]).
 * Reference pixels outside the frame are edge-replicated (the WRAP mode of
 * main/full_me.cu:41, checked by its clamp at :75-78).
 * mv receives (mv_y, mv_x, sad) int32 per block, blocks in raster order: the
 * minimum SAD, ties resolved to the first displacement in raster order of
 * (dy, dx).  b in {8, 16}; 1 <= r <= 64; pitch = w. */
umi_status umi_full_me_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b, int32_t r,
                          const int32_t* centers, int32_t* mv, void* stream);
/* The same search restricted to a device-side list of blocks: searches
 * blocks[0 .. *n_blocks) (block indices in raster order; *n_blocks is read on
 * the device, so it may be produced by an earlier kernel on the stream) and
 * writes their (mv_y, mv_x, sad) at their own positions of `mv`, leaving the
 * other entries untouched.  max_blocks bounds *n_blocks (grid size). */
umi_status umi_full_me_u8_list(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b, int32_t r,
                               const int32_t* centers, const int32_t* blocks, const int32_t* n_blocks,
                               int32_t max_blocks, int32_t* mv, void* stream);
/* Error word of the full-search kernels, no counterpart in the reference
 * (whose kernels have no bounded waits).  The searches of umi_full_me_u8 and
 * umi_full_me_u8_list at 16x16 blocks and r = 32 or 64 run a warp-specialised
 * kernel whose mbarrier waits are bounded (1 s); a wait that gives up ORs an
 * error bit into a library-wide device word and the blocks it did not finish
 * get sad = -1.  This call synchronises `stream`, stores the word in *bits
 * (if non-NULL), clears it and returns UMI_ERR_TIMEOUT if it was set. */
umi_status umi_full_me_error(int32_t* bits, void* stream);
/* The same search without the argmin: writes the whole SAD volume
 * (h/b, w/b, 2r+1, 2r+1) int32, the output layout of main/full_me.cu:55-62. */
umi_status umi_full_me_sad_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b, int32_t r,
                              int32_t* sad, void* stream);

/* ---- Learned motion proposal for 16x16 block motion estimation.
 * No counterpart in the reference (its full_me, main/full_me.cu, only does
 * exhaustive search); the exhaustive search above stays the fallback.
 * Network: the pair (cur, ref) box-averaged 4x4, (mean - 128) / 32 -> four 3x3 convolutions
 * (32 channels, dilations 1, 2, 4, 8, ReLU, bf16 weights, fp32 accumulation)
 * -> a linear head per 16x16 block over its 4x4 cells x 32 channels -> one
 * vector (mv_y, mv_x) / 16.  Parameters are one fp32 array of
 * umi_menet_param_count() floats: per layer the weights [cout][cin][3][3]
 * then the biases, then the head weights [2][32*4*4] (feature index
 * channel*16 + cell_row*4 + cell_col) and the head biases [2].
 * Frames are h x w uint8 with h, w multiples of 16 and pitch w.  All
 * pointers are device pointers; workspace is device memory of at least
 * umi_menet_workspace_bytes(h, w) bytes, 256-byte aligned. */
int32_t umi_menet_param_count(void);
size_t umi_menet_workspace_bytes(int32_t h, int32_t w);
/* Forward pass; keeps the activations in the workspace for
 * umi_menet_backward.  pred (may be NULL) receives (h/16 * w/16, 2) fp32. */
umi_status umi_menet_forward(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, const float* params,
                             float* pred, void* workspace, size_t workspace_bytes, void* stream);
/* Backward pass of the mean smooth-L1 loss between the last forward's
 * prediction and target/16 (target: int32 vectors (mv_y, mv_x) per block at
 * target[k*target_stride], target[k*target_stride+1]).  Writes the full
 * gradient (param_count floats) to grads and, when loss is not NULL, the
 * loss (one float, device). */
umi_status umi_menet_backward(const int32_t* target, int32_t target_stride, int32_t h, int32_t w, const float* params,
                              float* grads, float* loss, void* workspace, size_t workspace_bytes, void* stream);
/* Inference forward pass (the one umi_me_learned_u8 runs): layer 1 on the
 * FP32 pipe, layers 2-4 on the tensor cores (tcgen05, bf16 activations,
 * fp32 accumulation), activations rounded to bf16 after each ReLU; pred (may
 * be NULL) as umi_menet_forward.  err (device, may be NULL) receives error
 * bits of bounded waits that gave up (0 when all is well). */
umi_status umi_menet_infer(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, const float* params,
                           float* pred, int32_t* err, void* workspace, size_t workspace_bytes, void* stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8; step counts from 1). */
umi_status umi_menet_adam(float* params, const float* grads, float* m, float* v, int32_t step, float lr,
                          void* stream);
/* Learned motion estimation: inference pass (umi_menet_infer), search centres round(16 * pred)
 * clamped to +-(full_r - refine_r), exhaustive search in +-refine_r around
 * them.  Audit: when audit_stride > 0, blocks 0, audit_stride, 2*audit_stride,
 * ... are also searched exhaustively in +-full_r around (0, 0); they take
 * that exact result, and audit_sums (device, 2 x uint64, may be NULL)
 * receives the sum over them of the refined SAD and of the exhaustive SAD
 * (the sampled SAD regression is their ratio - 1).  Fallback: every other
 * block whose refined SAD exceeds sad_threshold is searched exhaustively in
 * +-full_r around (0, 0).  mv receives (mv_y, mv_x, sad) per block as
 * umi_full_me_u8 with b = 16; n_fallback (device, may be NULL) the number of
 * fallback blocks.  1 <= refine_r <= full_r <= 64.  The audit's exhaustive
 * search does not depend on the proposal: when it has at least as many
 * blocks as the GPU has SMs, it runs on a second stream of the calling host
 * thread (one per device, made on the first call outside a stream capture),
 * forked from `stream` at entry and joined back before the call's last work
 * on `stream`; stream order and capture are kept.  A smaller audit joins the
 * fallback blocks' exhaustive search. */
umi_status umi_me_learned_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, const float* params,
                             int32_t refine_r, int32_t full_r, int32_t sad_threshold, int32_t audit_stride,
                             int32_t* mv, unsigned long long* audit_sums, int32_t* n_fallback, void* workspace,
                             size_t workspace_bytes, void* stream);

/* Coarse-to-fine motion proposal (no reference counterpart; the fast
 * proposal beside the learned one).  Cells are rounded 4x4 means
 * q(img, y, x) = (sum_{u,v<4} img[clamp(y+u)][clamp(x+v)] + 8) >> 4.  For
 * every 16x16 block, centers (device, nblk x 2 int32) receives the even
 * displacement (dy, dx) in [-range, range]^2 minimising
 * sum_{i,j<4} |q(cur, 16by+4i, 16bx+4j) - q(ref, 16by+4i+dy, 16bx+4j+dx)|,
 * ties to the first in raster order of (dy, dx).  range even, 0..62; h, w
 * multiples of 16.  workspace: device, 256-byte aligned,
 * umi_me_coarse_workspace_bytes(h, w) bytes (0: frame unsupported). */
size_t umi_me_coarse_workspace_bytes(int32_t h, int32_t w);
umi_status umi_me_coarse_centers_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t range,
                                    int32_t* centers, void* workspace, size_t workspace_bytes, void* stream);
/* Motion estimation from the coarse proposal: centres as
 * umi_me_coarse_centers_u8 with range = (full_r - refine_r) rounded down to
 * even, then the refine, audit and fallback of umi_me_learned_u8 with the
 * same arguments and outputs. */
umi_status umi_me_coarse_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t refine_r,
                            int32_t full_r, int32_t sad_threshold, int32_t audit_stride, int32_t* mv,
                            unsigned long long* audit_sums, int32_t* n_fallback, void* workspace,
                            size_t workspace_bytes, void* stream);

/* Bilateral filter, float32 (h, w), (2*radius+1)^2 window, radius 1..3.
 * out = sum(w*n) / sum(w) with w = exp(-(n-c)^2 / (2 sigma_r^2)) *
 * ws[dy] * ws[dx], ws[i] = exp(-(i-radius)^2 / (2 sigma_s^2)), c the centre
 * pixel; neighbours outside the image read as 0 and still contribute.
 * Replaces the Execute call of main/bilateral.cu:54-100 (Bilateral strategy,
 * main/bilateral.cu:9-24: there the spatial weights are a memory and the
 * window is 25x25; the arithmetic per neighbour is the same). */
umi_status umi_bilateral_f32(const float* in, float* out, int32_t h, int32_t w, int32_t radius, float sigma_s,
                             float sigma_r, void* stream);

/* 3x3 filter with a weight per pixel: out[y,x] = sum_{dy,dx}
 * wts[y,x,dy+1,dx+1] * in[y+dy, x+dx], zero outside the image; wts is
 * (h, w, 3, 3) float32.  The per-pixel form of main/wfilter3x3.cu:39-69
 * (there the weight memory is one 3x3 kernel). */
umi_status umi_wfilter3x3_pp_f32(const float* in, const float* wts, float* out, int32_t h, int32_t w, void* stream);

/* Dot-product cost volume: left, right are (c, h, w) float32 feature maps,
 * cv is (h, w, nd) float32 with cv[y,x,d] = sum_ch left[ch,y,x] *
 * right[ch,y,x+d], right zero beyond the image.  nd in {16, 32, 64}.  The
 * dot-product form of the horizontal cost volume of main/cost_volume.cu:17-65
 * (there: |a-b| over a 7-tap window). */
umi_status umi_cost_volume_dot_f32(const float* left, const float* right, float* cv, int32_t c, int32_t h, int32_t w,
                                   int32_t nd, void* stream);

/* Tensor-core GEMM (tcgen05, sm_103a): C[M,N] = A[M,K] * B[N,K]^T with A and
 * B row-major bf16 (umi_gemm_bf16) or f16 (umi_gemm_f16), fp32 accumulation
 * and fp32 row-major C.  K must be a multiple of 8; A, B 16-byte aligned.
 * `err` (optional, device int) receives error bits if a bounded internal wait
 * gave up (then the call also leaves C unspecified); it is never cleared by the
 * library.  Replaces the Execute call of main/gemm.cu:37-67 (Gemm strategy,
 * main/gemm.cu:8-15) for half-precision operands; note B is taken transposed
 * (N x K), the layout both tensor-core operands share. */
umi_status umi_gemm_bf16(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t* err,
                         void* stream);
umi_status umi_gemm_f16(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t* err,
                        void* stream);
/* Failure-path hook, no counterpart in the reference: umi_gemm_bf16 with the
 * epilogue's bounded wait for each finished accumulator limited to
 * epilogue_wait_ns nanoseconds instead of 1 s.  A limit shorter than one
 * tile's MMAs makes that wait give up: the kernel records error bit 4 in
 * *err, every role stops, the producer's copies and the issued MMAs drain,
 * TMEM is freed and the kernel returns (C is then unspecified), leaving the
 * context usable.  Used by the tests of the timeout path. */
umi_status umi_gemm_bf16_wait_limit(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K,
                                    int32_t* err, unsigned long long epilogue_wait_ns, void* stream);
/* Maps the error bits a kernel left in its `err` word (read back by the
 * caller after the stream finished) to a status: UMI_OK for 0, else
 * UMI_ERR_TIMEOUT with the bits named in umi_last_error_string(). */
umi_status umi_err_status(int32_t err_bits);
/* FP32 GEMM emulated on the bf16 tensor cores by operand splitting (bf16x3:
 * A = A_hi + A_lo, B = B_hi + B_lo, C = A_hi B_hi + A_lo B_hi + A_hi B_lo, fp32
 * accumulation; Henry, Tang & Heinecke, ARITH 2019).  A is (M,K), B is (N,K),
 * both fp32 row-major.  Needs a workspace of
 * umi_gemm_f32_bf16x3_workspace_bytes(M, N, K) bytes (256-byte aligned) for the
 * split operands. */
size_t umi_gemm_f32_bf16x3_workspace_bytes(int32_t M, int32_t N, int32_t K);
umi_status umi_gemm_f32_bf16x3(const float* A, const float* B, float* C, int32_t M, int32_t N, int32_t K,
                               void* workspace, size_t workspace_bytes, int32_t* err, void* stream);
/* FP32 GEMM at FP32-level accuracy on the f16 tensor cores: operand
 * splitting with error correction (Ootomo & Yokota, IJHPCA 2022):
 * x = x_hi + 2^-11 x_lo (x_hi = rn_f16(x), x_lo = rn_f16((x - x_hi) 2^11)),
 * C = A_hi B_hi^T + 2^-11 (A_hi B_lo^T + A_lo B_hi^T).  The tensor core's
 * fp32 accumulation truncates, so A_hi B_hi is accumulated in tensor memory
 * for `chunk` K-slices of 64 only (0: default 2) and each chunk is added into
 * fp32 registers with round-to-nearest adds.  A (M,K) and B (N,K) fp32
 * row-major, 16-byte aligned, K a multiple of 8, |values| < 65504.  Needs a
 * workspace of umi_gemm_f32_f16x3_workspace_bytes(M, N, K) bytes (256-byte
 * aligned) for the split operands.  `err` as for umi_gemm_bf16.  Replaces the
 * Execute call of main/gemm.cu:37-67 (Gemm strategy, main/gemm.cu:8-15) for
 * fp32 operands. */
size_t umi_gemm_f32_f16x3_workspace_bytes(int32_t M, int32_t N, int32_t K);
umi_status umi_gemm_f32_f16x3(const float* A, const float* B, float* C, int32_t M, int32_t N, int32_t K, int32_t chunk,
                              void* workspace, size_t workspace_bytes, int32_t* err, void* stream);

/* Convolution forward pass on the tensor cores (implicit GEMM, tcgen05):
 * out[n,k,y,x] = sum_{c,dy,dx} w[k,dy,dx,c] * in[n,y+dy-r/2,x+dx-r/2,c], stride
 * 1, zero padding r/2 (same size output).  in is NHWC bf16, w is KRSC bf16,
 * out is NCHW fp32 (fp32 accumulation).  c a multiple of 64, r in {1,3,5,7},
 * 16-byte aligned inputs.  `err` as for umi_gemm_bf16.  The tensor-core form
 * of the direct convolution of main/fprop.cu:53-82 (Gemm strategy over
 * (N, K, OH, OW) x (C, R, S); there int32, stride 2, 7x7). */
umi_status umi_conv2d_fprop_bf16(const void* x_nhwc, const void* w_krsc, float* out_nchw, int32_t n, int32_t c,
                                 int32_t h, int32_t w, int32_t k, int32_t r, int32_t* err, void* stream);
/* The same convolution on fp32 input and weights at FP32-level accuracy: the
 * split of umi_gemm_f32_f16x3 applied to the implicit GEMM (x NHWC fp32, w
 * KRSC fp32, out NCHW fp32; c a multiple of 64; r in 1, 3, 5, 7).  Needs a
 * workspace of umi_conv2d_fprop_f32_f16x3_workspace_bytes(...) bytes
 * (256-byte aligned).  `chunk` and `err` as for umi_gemm_f32_f16x3.
 * Replaces the Execute call of main/fprop.cu:49-82 for fp32 data. */
size_t umi_conv2d_fprop_f32_f16x3_workspace_bytes(int32_t n, int32_t c, int32_t h, int32_t w, int32_t k, int32_t r);
umi_status umi_conv2d_fprop_f32_f16x3(const float* x_nhwc, const float* w_krsc, float* out_nchw, int32_t n, int32_t c,
                                      int32_t h, int32_t w, int32_t k, int32_t r, int32_t chunk, void* workspace,
                                      size_t workspace_bytes, int32_t* err, void* stream);

/* ---- batched launches: many images of uneven sizes in one persistent
 * launch.  The image table is copied into the launch (no device allocation);
 * CTAs walk a prefix-summed queue of tiles across all images.  `variant`
 * selects a tile shape (0 .. umi_batch_variants(op)-1; -1 = default), as
 * chosen by umi_autotune_batch.  The reference launches once per image and
 * allocates its index tables per call (src/UMI_gpu.h:374-381). */
#define UMI_BATCH_MAX_IMAGES 256
typedef enum { UMI_OP_BILATERAL = 0, UMI_OP_WFILTER_PP = 1, UMI_OP_COST_VOLUME = 2 } umi_batch_op;
typedef struct {
	const float* in;   /* bilateral / wfilter: image; cost volume: left features */
	const float* aux;  /* wfilter: weights (h,w,3,3); cost volume: right features; else NULL */
	float* out;
	int32_t h, w;
} umi_batch_image;
typedef struct {
	int32_t radius;    /* bilateral */
	float sigma_s, sigma_r;
	int32_t channels;  /* cost volume */
	int32_t nd;        /* cost volume */
} umi_batch_params;

int32_t umi_batch_variants(int32_t op);
umi_status umi_batch_run(int32_t op, const umi_batch_image* images, int32_t n_images, const umi_batch_params* params,
                         int32_t variant, void* stream);
/* Times every variant of `op` on this batch (CUDA events, `reps` launches
 * each after one warm-up) and returns the fastest in *best_variant and its
 * time in *best_ms.  The batch's outputs are overwritten. */
umi_status umi_autotune_batch(int32_t op, const umi_batch_image* images, int32_t n_images,
                              const umi_batch_params* params, int32_t reps, int32_t* best_variant, float* best_ms,
                              void* stream);

/* Batch graphs: a sequence of batched launches recorded once into a CUDA
 * graph and replayed by one call.  umi_batch_graph_add records
 * umi_batch_run(op, images, n_images, params, variant) after the previous
 * ones (the image table is copied at that moment: later replays use the same
 * buffers); umi_batch_graph_launch replays the whole sequence on `stream`
 * (instantiating the graph on first use).  The handle owns host-side CUDA
 * objects only; destroy it when no replay is pending.  The reference has no
 * batching (one Execute per image). */
typedef struct umi_batch_graph umi_batch_graph;
umi_status umi_batch_graph_create(umi_batch_graph** graph);
umi_status umi_batch_graph_add(umi_batch_graph* graph, int32_t op, const umi_batch_image* images, int32_t n_images,
                               const umi_batch_params* params, int32_t variant);
/* One launch for a whole batch step, no counterpart in the reference (which
 * runs one Execute per image and operator): up to one job per operator
 * (bilateral, per-pixel-weight filter, dot-product cost volume), each with its
 * images, parameters and, per image, the variant that serves it (tile shape
 * and pixels per thread; NULL: variant 0 for every image; see
 * umi_batch_fused_variants).  One persistent kernel walks every CTA's share of
 * the cost-volume tiles (tensor cores), then of one queue holding the two
 * filters' tiles of all images.  The cost-volume job must use nd = 64, 1..32
 * channels and 16-byte aligned outputs (else UMI_ERR_UNSUPPORTED: use
 * umi_batch_run per operator); at most UMI_BATCH_MAX_IMAGES images in each
 * job and in the filters' queue together.  Allocates nothing. */
typedef struct {
	int32_t op; /* umi_batch_op */
	const umi_batch_image* images;
	int32_t n_images;
	umi_batch_params params;
	const int32_t* variants; /* n_images host ints, or NULL */
} umi_batch_job;
int32_t umi_batch_fused_variants(int32_t op);
umi_status umi_batch_run_fused(const umi_batch_job* jobs, int32_t n_jobs, void* stream);
/* Records one umi_batch_run_fused launch as the next node of `graph`. */
umi_status umi_batch_graph_add_fused(umi_batch_graph* graph, const umi_batch_job* jobs, int32_t n_jobs);
umi_status umi_batch_graph_launch(umi_batch_graph* graph, void* stream);
void umi_batch_graph_destroy(umi_batch_graph* graph);

#ifdef __cplusplus
}
#endif
#endif /* UMI_GB300_H */
