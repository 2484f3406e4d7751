/* CPU oracle for the UMI operator hot path: closed-form scalar restatements.
 *
 * TEST INFRASTRUCTURE ONLY.  These functions are the checker for the GPU
 * kernels and the timed CPU baseline; the product path never calls them.
 *
 * Two groups:
 *  1. oracle_ref_*: the scalar CPU loops with which each example program of
 *     johnjohnlin/UMI checks its GPU result (main/<app>.cu, lines cited per
 *     function), restated in C with the same arithmetic and the same types.
 *  2. oracle_*: the same operators at the sizes and element types of the
 *     benchmark workloads (uint8 frames, float images), with FP64
 *     accumulation for the floating-point ones.
 * Every function is deterministic; `threads` <= 0 means "all OpenMP threads".
 */
#ifndef UMI_ORACLE_H
#define UMI_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- group 1: the reference's own CPU checks (int32 / float) ---- */
/* main/filter3x3.cu:60-78 */
void oracle_ref_filter3x3_i32(const int32_t* in, int32_t* out, int h, int w, int init, int mul, int pad);
/* main/wfilter3x3.cu:71-89 */
void oracle_ref_wfilter3x3_i32(const int32_t* in, int32_t* out, int h, int w, const int32_t* w9, int init, int pad);
/* main/bilateral.cu:103-123 (float arithmetic, expf, as written) */
void oracle_ref_bilateral_f32(const float* in, float* out, int h, int w, int ofs, const float* ws, float norm);
/* main/cost_volume.cu:67-80: out is (h, w, sr) */
void oracle_ref_cost_volume_i32(const int32_t* frame, int32_t* cv, int h, int w, int k, int sr);
/* main/full_me.cu:66-87, generalised to a (cur, ref) pair; out is
 * (h/b, w/b, sr, sr) with displacement (sy, sx) + sr_ofs */
void oracle_ref_full_me_i32(const int32_t* cur, const int32_t* ref, int32_t* sad, int h, int w, int b, int sr_ofs, int sr);
/* main/iimg.cu:84-112 (row prefix then column prefix) */
void oracle_ref_iimg_i32(const int32_t* in, int32_t* out, int h, int w);
/* main/gemm.cu:69-78 */
void oracle_ref_gemm_i32(const int32_t* A, const int32_t* B, int32_t* C, int m, int k, int n);
/* main/fprop.cu:84-108: NCHW input, KCff weights, (N, K, ih/s, iw/s) output */
void oracle_ref_fprop_i32(const int32_t* in, const int32_t* wt, int32_t* out, int n, int c, int ih, int iw,
                          int k, int f, int s, int ofs, int threads);
/* Inputs of main/fprop.cu:41-47: std::default_random_engine (default seed)
 * feeding uniform_int_distribution<int>(0, 10), first the input then the
 * weights. */
void oracle_ref_fprop_inputs(int32_t* in, size_t n_in, int32_t* wt, size_t n_wt);

/* ---- group 2: benchmark workloads ---- */
/* 3x3 weighted filter, zero padding value `pad`, FP64 accumulation in the
 * order (dy, dx) row-major. */
void oracle_filter3x3_f64(const float* in, double* out, int h, int w, const float* w9, float pad, int threads);
/* Integral image uint8 -> int32 (inclusive in both axes). */
void oracle_iimg_u8_i32(const uint8_t* in, int32_t* out, int h, int w, int threads);
/* Full-search block motion estimation, uint8 frames, block b x b, search
 * [-r, r]^2, edge-replicated (clamped) reference, blocks truncated at the
 * frame edge (h/b x w/b).  For each block writes (mv_y, mv_x, sad): the
 * minimum SAD, ties broken by the first displacement in raster order of
 * (dy, dx) starting at (-r, -r).  If `blocks` is non-NULL only the n_blocks
 * listed block indices (by*nbx + bx) are searched and written (in list
 * order, 3 ints each).  `sad_volume`, when non-NULL, receives the whole
 * (nby, nbx, 2r+1, 2r+1) SAD volume (only valid with blocks == NULL). */
void oracle_full_me_u8(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int r,
                       const int32_t* blocks, int n_blocks, int32_t* mv, int32_t* sad_volume, int threads);
/* The reference's CPU loop for full_me (main/full_me.cu:68-87) as written:
 * every reference pixel clamped individually, int arithmetic, on uint8
 * frames, plus the argmin; blocks[i] selects the searched blocks.  This is
 * the timed CPU baseline (not a checker: oracle_full_me_u8 is faster). */
void oracle_ref_full_me_u8_argmin(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int r,
                                  const int32_t* blocks, int n_blocks, int32_t* mv, int threads);
/* The reference's iimg loop (main/iimg.cu:100-111) on a uint8 frame:
 * row prefix into out, then column prefix in place (timed CPU baseline). */
void oracle_ref_iimg_u8(const uint8_t* in, int32_t* out, int h, int w);
/* Coarse motion proposal (no reference counterpart).  Cells are rounded 4x4
 * means q(img, y, x) = (sum_{u,v<4} img[clamp(y+u)][clamp(x+v)] + 8) >> 4.
 * For every 16x16 block (h/16 x w/16, row-major) writes centers[2 blk ..] =
 * the even displacement (dy, dx) in [-range, range]^2 minimising
 * sum_{i,j<4} |q(cur, 16by+4i, 16bx+4j) - q(ref, 16by+4i+dy, 16bx+4j+dx)|,
 * ties to the first in raster order of (dy, dx).  range is even. */
void oracle_coarse_centers_u8(const uint8_t* cur, const uint8_t* ref, int h, int w, int range, int32_t* centers,
                              int threads);
/* SAD of one block at one displacement (same clamping rule). */
int32_t oracle_block_sad_u8(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int by, int bx, int dy, int dx);
/* Bilateral filter, (2r+1)^2 window, spatial weight exp(-d^2/(2 s_s^2)) per
 * axis, range weight exp(-(n-c)^2/(2 s_r^2)); neighbours outside the image
 * read as 0 and still contribute (main/bilateral.cu:72,111-117).  FP64. */
void oracle_bilateral_f64(const float* in, double* out, int h, int w, int r, double sigma_s, double sigma_r, int threads);
/* Per-pixel weighted 3x3 filter: wts is (h, w, 3, 3), zero padding. FP64. */
void oracle_wfilter_pp_f64(const float* in, const float* wts, double* out, int h, int w, int threads);
/* Dot-product cost volume: L, R are (c, h, w); cv is (h, w, nd) with
 * cv[y,x,d] = sum_c L[c,y,x] * R[c,y,x+d], R zero outside the image. FP64. */
void oracle_cost_volume_dot_f64(const float* L, const float* R, double* cv, int c, int h, int w, int nd, int threads);
/* C[m,n] = sum_k A[m,k] B[k,n] (row-major), FP64 accumulation of the given
 * float operands. If b_is_nk, B is stored (n, k). */
void oracle_gemm_f64(const float* A, const float* B, double* C, int m, int n, int k, int b_is_nk, int threads);
/* 2-D convolution (cross-correlation), NCHW input, KCRS weights, stride s,
 * zero padding p, FP64. out is (n, k, oh, ow). */
void oracle_conv2d_f64(const float* in, const float* wt, double* out, int n, int c, int h, int w, int k, int r,
                       int s, int p, int threads);

#ifdef __cplusplus
}
#endif
#endif
