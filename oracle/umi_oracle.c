/* CPU oracle for the UMI operator hot path.  TEST INFRASTRUCTURE ONLY: the
 * checker for the GPU kernels and the timed CPU baseline.  See umi_oracle.h
 * for the contract of each function and the reference lines it restates. */
#include "umi_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static int nthreads(int t) {
#ifdef _OPENMP
	return t > 0 ? t : omp_get_max_threads();
#else
	(void)t;
	return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* group 1: the reference's own CPU checks                             */
/* ------------------------------------------------------------------ */

/* main/filter3x3.cu:60-78: sum of the 3x3 neighbourhood starting from init,
 * out-of-image neighbours contribute `pad`, result times mul. */
void oracle_ref_filter3x3_i32(const int32_t* in, int32_t* out, int h, int w, int init, int mul, int pad) {
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x) {
			int32_t s = init;
			for (int dy = -1; dy <= 1; ++dy)
				for (int dx = -1; dx <= 1; ++dx) {
					int yy = y + dy, xx = x + dx;
					s += (yy < 0 || yy >= h || xx < 0 || xx >= w) ? pad : in[(size_t)w * yy + xx];
				}
			out[(size_t)w * y + x] = s * mul;
		}
}

/* main/wfilter3x3.cu:71-89: weighted 3x3 sum, weights row-major (dy, dx). */
void oracle_ref_wfilter3x3_i32(const int32_t* in, int32_t* out, int h, int w, const int32_t* w9, int init, int pad) {
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x) {
			int32_t s = init;
			for (int dy = -1; dy <= 1; ++dy)
				for (int dx = -1; dx <= 1; ++dx) {
					int yy = y + dy, xx = x + dx;
					int32_t wt = w9[3 * (dy + 1) + (dx + 1)];
					s += wt * ((yy < 0 || yy >= h || xx < 0 || xx >= w) ? pad : in[(size_t)w * yy + xx]);
				}
			out[(size_t)w * y + x] = s;
		}
}

/* main/bilateral.cu:103-123: neighbours outside the image read as 0.0 and
 * still contribute to both sums; float arithmetic with expf. */
void oracle_ref_bilateral_f32(const float* in, float* out, int h, int w, int ofs, const float* ws, float norm) {
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x) {
			float wsum = 0.0f, wxsum = 0.0f;
			const float cur = in[(size_t)w * y + x];
			for (int dy = -ofs; dy <= ofs; ++dy)
				for (int dx = -ofs; dx <= ofs; ++dx) {
					int yy = y + dy, xx = x + dx;
					float n = 0.0f;
					if (xx >= 0 && xx < w && yy >= 0 && yy < h) n = in[(size_t)w * yy + xx];
					float d = n - cur;
					float wt = expf(d * d * norm) * ws[dy + ofs] * ws[dx + ofs];
					wsum += wt;
					wxsum += wt * n;
				}
			out[(size_t)w * y + x] = wxsum / wsum;
		}
}

/* main/cost_volume.cu:67-80: horizontal SAD over a k-tap window, sr offsets
 * centred on 0, both taps clamped to the row. */
void oracle_ref_cost_volume_i32(const int32_t* f, int32_t* cv, int h, int w, int k, int sr) {
	const int ko = k / 2, so = sr / 2;
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x)
			for (int sx = -so; sx <= so; ++sx) {
				int32_t sad = 0;
				for (int t = -ko; t <= ko; ++t) {
					int rx = clampi(x + t, 0, w - 1), qx = clampi(x + sx + t, 0, w - 1);
					sad += abs(f[(size_t)y * w + rx] - f[(size_t)y * w + qx]);
				}
				cv[((size_t)y * w + x) * sr + (sx + so)] = sad;
			}
}

/* main/full_me.cu:66-87 with separate current / reference frames. */
void oracle_ref_full_me_i32(const int32_t* cur, const int32_t* ref, int32_t* sad, int h, int w, int b, int sr_ofs, int sr) {
	size_t c = 0;
	for (int y = 0; y + b <= h; y += b)
		for (int x = 0; x + b <= w; x += b)
			for (int sy = 0; sy < sr; ++sy)
				for (int sx = 0; sx < sr; ++sx) {
					int32_t s = 0;
					for (int py = 0; py < b; ++py)
						for (int px = 0; px < b; ++px) {
							int spy = clampi(y + py + sy + sr_ofs, 0, h - 1);
							int spx = clampi(x + px + sx + sr_ofs, 0, w - 1);
							s += abs(cur[(size_t)(y + py) * w + (x + px)] - ref[(size_t)spy * w + spx]);
						}
					sad[c++] = s;
				}
}

/* main/iimg.cu:100-111: row prefix sums, then column prefix sums. */
void oracle_ref_iimg_i32(const int32_t* in, int32_t* out, int h, int w) {
	for (int y = 0; y < h; ++y) {
		int32_t s = 0;
		for (int x = 0; x < w; ++x) out[(size_t)w * y + x] = s += in[(size_t)w * y + x];
	}
	for (int x = 0; x < w; ++x) {
		int32_t s = 0;
		for (int y = 0; y < h; ++y) out[(size_t)w * y + x] = s += out[(size_t)w * y + x];
	}
}

/* main/gemm.cu:69-78 */
void oracle_ref_gemm_i32(const int32_t* A, const int32_t* B, int32_t* C, int m, int k, int n) {
	for (int y = 0; y < m; ++y)
		for (int x = 0; x < n; ++x) {
			int32_t s = 0;
			for (int t = 0; t < k; ++t) s += A[(size_t)y * k + t] * B[(size_t)t * n + x];
			C[(size_t)y * n + x] = s;
		}
}

/* main/fprop.cu:84-108: direct convolution, zero outside the input. */
void oracle_ref_fprop_i32(const int32_t* in, const int32_t* wt, int32_t* out, int n, int c, int ih, int iw,
                          int k, int f, int s, int ofs, int threads) {
	const int oh = ih / s, ow = iw / s;
#pragma omp parallel for collapse(2) num_threads(nthreads(threads)) schedule(static)
	for (int i = 0; i < n; ++i)
		for (int oc = 0; oc < k; ++oc)
			for (int oy = 0; oy < oh; ++oy)
				for (int ox = 0; ox < ow; ++ox) {
					int32_t sum = 0;
					const int iy = oy * s, ix = ox * s;
					for (int ic = 0; ic < c; ++ic)
						for (int dy = 0; dy < f; ++dy)
							for (int dx = 0; dx < f; ++dx) {
								int xx = ix + dx + ofs, yy = iy + dy + ofs;
								int32_t wv = wt[(((size_t)oc * c + ic) * f + dy) * f + dx];
								if (0 <= xx && xx < iw && 0 <= yy && yy < ih)
									sum += wv * in[(((size_t)i * c + ic) * ih + yy) * iw + xx];
							}
					out[(((size_t)i * k + oc) * oh + oy) * ow + ox] = sum;
				}
}

/* ------------------------------------------------------------------ */
/* group 2: benchmark workloads                                        */
/* ------------------------------------------------------------------ */

void oracle_filter3x3_f64(const float* in, double* out, int h, int w, const float* w9, float pad, int threads) {
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x) {
			double s = 0.0;
			for (int dy = -1; dy <= 1; ++dy)
				for (int dx = -1; dx <= 1; ++dx) {
					int yy = y + dy, xx = x + dx;
					double v = (yy < 0 || yy >= h || xx < 0 || xx >= w) ? (double)pad : (double)in[(size_t)w * yy + xx];
					s += (double)w9[3 * (dy + 1) + (dx + 1)] * v;
				}
			out[(size_t)w * y + x] = s;
		}
}

void oracle_iimg_u8_i32(const uint8_t* in, int32_t* out, int h, int w, int threads) {
	(void)threads;
	for (int y = 0; y < h; ++y) {
		int32_t s = 0;
		for (int x = 0; x < w; ++x) {
			s += in[(size_t)w * y + x];
			out[(size_t)w * y + x] = s + (y ? out[(size_t)w * (y - 1) + x] : 0);
		}
	}
}

int32_t oracle_block_sad_u8(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int by, int bx, int dy, int dx) {
	const int y0 = by * b, x0 = bx * b;
	int32_t s = 0;
	if (y0 + dy >= 0 && y0 + dy + b <= h && x0 + dx >= 0 && x0 + dx + b <= w) {
		for (int py = 0; py < b; ++py) {
			const uint8_t* c = cur + (size_t)(y0 + py) * w + x0;
			const uint8_t* r = ref + (size_t)(y0 + py + dy) * w + x0 + dx;
			for (int px = 0; px < b; ++px) s += abs((int)c[px] - (int)r[px]);
		}
		return s;
	}
	for (int py = 0; py < b; ++py) {
		const int ry = clampi(y0 + py + dy, 0, h - 1);
		for (int px = 0; px < b; ++px) {
			const int rx = clampi(x0 + px + dx, 0, w - 1);
			s += abs((int)cur[(size_t)(y0 + py) * w + x0 + px] - (int)ref[(size_t)ry * w + rx]);
		}
	}
	return s;
}

void oracle_full_me_u8(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int r,
                       const int32_t* blocks, int n_blocks, int32_t* mv, int32_t* sad_volume, int threads) {
	const int nby = h / b, nbx = w / b, nd = 2 * r + 1;
	const int total = blocks ? n_blocks : nby * nbx;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 4)
	for (int i = 0; i < total; ++i) {
		const int blk = blocks ? blocks[i] : i;
		const int by = blk / nbx, bx = blk % nbx;
		int32_t best = 0x7fffffff, bdy = 0, bdx = 0;
		for (int dy = -r; dy <= r; ++dy)
			for (int dx = -r; dx <= r; ++dx) {
				const int32_t s = oracle_block_sad_u8(cur, ref, h, w, b, by, bx, dy, dx);
				if (sad_volume && !blocks)
					sad_volume[((size_t)blk * nd + (dy + r)) * nd + (dx + r)] = s;
				if (s < best) { best = s; bdy = dy; bdx = dx; }
			}
		mv[3 * (size_t)i + 0] = bdy;
		mv[3 * (size_t)i + 1] = bdx;
		mv[3 * (size_t)i + 2] = best;
	}
}

static int box_q(const uint8_t* img, int h, int w, int y, int x) {
	int s = 0;
	for (int u = 0; u < 4; ++u) {
		const uint8_t* row = img + (size_t)clampi(y + u, 0, h - 1) * w;
		for (int v = 0; v < 4; ++v) s += row[clampi(x + v, 0, w - 1)];
	}
	return (s + 8) >> 4;
}

void oracle_coarse_centers_u8(const uint8_t* cur, const uint8_t* ref, int h, int w, int range, int32_t* centers,
                              int threads) {
	const int nby = h / 16, nbx = w / 16, m = range / 2;
	/* q(ref) at every even position (2 y2, 2 x2) a block's candidates reach:
	 * y2 = 8 by + 2 i + dy/2 in [-m, 8 nby + m) */
	const int qh = 8 * nby + 2 * m, qw = 8 * nbx + 2 * m;
	int* q = (int*)malloc(sizeof(int) * (size_t)qh * qw);
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int y2 = 0; y2 < qh; ++y2)
		for (int x2 = 0; x2 < qw; ++x2) q[(size_t)y2 * qw + x2] = box_q(ref, h, w, 2 * (y2 - m), 2 * (x2 - m));
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 4)
	for (int blk = 0; blk < nby * nbx; ++blk) {
		const int by = blk / nbx, bx = blk % nbx;
		int c[16];
		for (int i = 0; i < 4; ++i)
			for (int j = 0; j < 4; ++j) c[4 * i + j] = box_q(cur, h, w, 16 * by + 4 * i, 16 * bx + 4 * j);
		int best = 0x7fffffff, bdy = 0, bdx = 0;
		for (int dy2 = -m; dy2 <= m; ++dy2)
			for (int dx2 = -m; dx2 <= m; ++dx2) {
				int s = 0;
				for (int i = 0; i < 4; ++i)
					for (int j = 0; j < 4; ++j)
						s += abs(c[4 * i + j] - q[(size_t)(8 * by + 2 * i + dy2 + m) * qw + (8 * bx + 2 * j + dx2 + m)]);
				if (s < best) { best = s; bdy = 2 * dy2; bdx = 2 * dx2; }
			}
		centers[2 * (size_t)blk] = bdy;
		centers[2 * (size_t)blk + 1] = bdx;
	}
	free(q);
}

void oracle_ref_full_me_u8_argmin(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int r,
                                  const int32_t* blocks, int n_blocks, int32_t* mv, int threads) {
	const int nbx = w / b;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 1)
	for (int i = 0; i < n_blocks; ++i) {
		const int y = (blocks[i] / nbx) * b, x = (blocks[i] % nbx) * b;
		int best = 0x7fffffff, bdy = 0, bdx = 0;
		for (int sy = -r; sy <= r; ++sy)
			for (int sx = -r; sx <= r; ++sx) {
				int sum = 0;
				for (int py = 0; py < b; ++py)
					for (int px = 0; px < b; ++px) {
						int spy = y + py + sy, spx = x + px + sx;
						spy = spy > h - 1 ? h - 1 : spy; spy = spy < 0 ? 0 : spy;
						spx = spx > w - 1 ? w - 1 : spx; spx = spx < 0 ? 0 : spx;
						sum += abs((int)cur[(size_t)(y + py) * w + (x + px)] - (int)ref[(size_t)spy * w + spx]);
					}
				if (sum < best) { best = sum; bdy = sy; bdx = sx; }
			}
		mv[3 * (size_t)i] = bdy; mv[3 * (size_t)i + 1] = bdx; mv[3 * (size_t)i + 2] = best;
	}
}

void oracle_ref_iimg_u8(const uint8_t* in, int32_t* out, int h, int w) {
	for (int y = 0; y < h; ++y) {
		int32_t s = 0;
		for (int x = 0; x < w; ++x) out[(size_t)w * y + x] = s += in[(size_t)w * y + x];
	}
	for (int x = 0; x < w; ++x) {
		int32_t s = 0;
		for (int y = 0; y < h; ++y) out[(size_t)w * y + x] = s += out[(size_t)w * y + x];
	}
}

void oracle_bilateral_f64(const float* in, double* out, int h, int w, int r, double sigma_s, double sigma_r, int threads) {
	double ws[64];
	for (int i = -r; i <= r; ++i) ws[i + r] = exp(-(double)(i * i) / (2.0 * sigma_s * sigma_s));
	const double nr = -1.0 / (2.0 * sigma_r * sigma_r);
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x) {
			const double c = in[(size_t)w * y + x];
			double sw = 0.0, swx = 0.0;
			for (int dy = -r; dy <= r; ++dy)
				for (int dx = -r; dx <= r; ++dx) {
					int yy = y + dy, xx = x + dx;
					double n = (yy < 0 || yy >= h || xx < 0 || xx >= w) ? 0.0 : (double)in[(size_t)w * yy + xx];
					double d = n - c;
					double wt = exp(d * d * nr) * ws[dy + r] * ws[dx + r];
					sw += wt;
					swx += wt * n;
				}
			out[(size_t)w * y + x] = swx / sw;
		}
}

void oracle_wfilter_pp_f64(const float* in, const float* wts, double* out, int h, int w, int threads) {
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x) {
			double s = 0.0;
			const float* wp = wts + ((size_t)y * w + x) * 9;
			for (int dy = -1; dy <= 1; ++dy)
				for (int dx = -1; dx <= 1; ++dx) {
					int yy = y + dy, xx = x + dx;
					double v = (yy < 0 || yy >= h || xx < 0 || xx >= w) ? 0.0 : (double)in[(size_t)w * yy + xx];
					s += (double)wp[3 * (dy + 1) + (dx + 1)] * v;
				}
			out[(size_t)w * y + x] = s;
		}
}

void oracle_cost_volume_dot_f64(const float* L, const float* R, double* cv, int c, int h, int w, int nd, int threads) {
	const size_t plane = (size_t)h * w;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int y = 0; y < h; ++y)
		for (int x = 0; x < w; ++x)
			for (int d = 0; d < nd; ++d) {
				double s = 0.0;
				if (x + d < w)
					for (int ch = 0; ch < c; ++ch)
						s += (double)L[ch * plane + (size_t)y * w + x] * (double)R[ch * plane + (size_t)y * w + x + d];
				cv[((size_t)y * w + x) * nd + d] = s;
			}
}

void oracle_gemm_f64(const float* A, const float* B, double* C, int m, int n, int k, int b_is_nk, int threads) {
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int i = 0; i < m; ++i) {
		double* crow = C + (size_t)i * n;
		for (int j = 0; j < n; ++j) crow[j] = 0.0;
		if (b_is_nk) {
			for (int j = 0; j < n; ++j) {
				double s = 0.0;
				for (int t = 0; t < k; ++t) s += (double)A[(size_t)i * k + t] * (double)B[(size_t)j * k + t];
				crow[j] = s;
			}
		} else {
			for (int t = 0; t < k; ++t) {
				const double a = A[(size_t)i * k + t];
				const float* brow = B + (size_t)t * n;
				for (int j = 0; j < n; ++j) crow[j] += a * (double)brow[j];
			}
		}
	}
}

void oracle_conv2d_f64(const float* in, const float* wt, double* out, int n, int c, int h, int w, int k, int r,
                       int s, int p, int threads) {
	const int oh = (h + 2 * p - r) / s + 1, ow = (w + 2 * p - r) / s + 1;
#pragma omp parallel for collapse(2) num_threads(nthreads(threads)) schedule(static)
	for (int i = 0; i < n; ++i)
		for (int oc = 0; oc < k; ++oc)
			for (int oy = 0; oy < oh; ++oy)
				for (int ox = 0; ox < ow; ++ox) {
					double sum = 0.0;
					for (int ic = 0; ic < c; ++ic)
						for (int dy = 0; dy < r; ++dy) {
							const int yy = oy * s + dy - p;
							if (yy < 0 || yy >= h) continue;
							for (int dx = 0; dx < r; ++dx) {
								const int xx = ox * s + dx - p;
								if (xx < 0 || xx >= w) continue;
								sum += (double)wt[(((size_t)oc * c + ic) * r + dy) * r + dx] *
								       (double)in[(((size_t)i * c + ic) * h + yy) * w + xx];
							}
						}
					out[(((size_t)i * k + oc) * oh + oy) * ow + ox] = sum;
				}
}
