// GPU drop-in check: the eight example applications of the reference
// (johnjohnlin/UMI main/*.cu) expressed through the source-compatible API,
// run on the GPU through UMI::Execute (include/umi/UMI_gpu.h).
//
// Each application uses the descriptors and inputs of the reference program
// (cited per app) and writes every output to <outdir>/<app>.<call>.bin;
// tests/test_gpu_dropin.py compares them with the digests in
// tests/golden/refpin.json (outputs the reference's own checks accepted).
// One JSON line per call reports the CUDA-event time of the Execute call.
//
// Usage: dropin_apps <outdir> [app]
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "umi/UMI_gpu.h"

using namespace UMI;

namespace {

std::string g_dir;
int g_fail = 0;

template <class T>
struct DevBuf {
	T* d = nullptr;
	size_t n = 0;
	explicit DevBuf(size_t n_) : n(n_) {
		cudaMalloc(&d, n * sizeof(T));
		cudaMemset(d, 0, n * sizeof(T));
	}
	DevBuf(const std::vector<T>& h) : DevBuf(h.size()) { cudaMemcpy(d, h.data(), n * sizeof(T), cudaMemcpyHostToDevice); }
	~DevBuf() { cudaFree(d); }
	std::vector<T> get() const {
		std::vector<T> h(n);
		cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
		return h;
	}
};

template <class T>
void dump(const std::string& app, int call, const DevBuf<T>& b) {
	const auto h = b.get();
	const std::string path = g_dir + "/" + app + "." + std::to_string(call) + ".bin";
	FILE* f = std::fopen(path.c_str(), "wb");
	if (!f) { ++g_fail; return; }
	std::fwrite(h.data(), sizeof(T), h.size(), f);
	std::fclose(f);
}

// Times one Execute call (CUDA events on the default stream) and checks it.
void timed(const char* app, int call, const std::function<umi_status()>& fn) {
	cudaEvent_t a, b;
	cudaEventCreate(&a);
	cudaEventCreate(&b);
	fn();  // warm-up (first launch loads the module)
	cudaDeviceSynchronize();
	cudaEventRecord(a);
	const umi_status st = fn();
	cudaEventRecord(b);
	const cudaError_t e = cudaDeviceSynchronize();
	float ms = 0;
	cudaEventElapsedTime(&ms, a, b);
	std::printf("{\"app\": \"%s\", \"call\": %d, \"status\": %d, \"cuda\": \"%s\", \"ms\": %.5f}\n", app, call, (int)st,
	            cudaGetErrorName(e), ms);
	if (st != UMI_OK || e != cudaSuccess) ++g_fail;
	cudaEventDestroy(a);
	cudaEventDestroy(b);
}

const auto PAD = PhysicalDim::PAD;
const auto WRAP = PhysicalDim::WRAP;

std::vector<int> iota_vec(size_t n) {
	std::vector<int> v(n);
	std::iota(v.begin(), v.end(), 0);
	return v;
}

// ---- main/filter3x3.cu:10-17 (strategy) and :19-58 (call) ----
struct NeighbourSum {
	int total;
	struct Constant { int init, mul; };
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = c.init; }
	STRATEGY_LOOP_STUB(1, 0) { total += IMEM(0, 0); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total * c.mul; }
};

void app_filter3x3() {
	const int w = 500, h = 300;
	DevBuf<int> in(iota_vec((size_t)w * h)), out((size_t)w * h);
	timed("filter3x3", 0, [&] {
		return Execute<NeighbourSum, 0x11, 0x1111, 0x1122>(
			{{{1, 1, 1, 1}, {1, 1, 1, 1}, {h, 16, 4, 1}, {w, 16, 8, 1}}},
			{{{1, 1}, {1, 1}, {3, 3}, {3, 3}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {{{}, {}, {2, -1, 1}, {3, -1, 1}}},
			   {{{1, PAD}, {1, PAD}, {h, PAD}, {w, PAD}}}, DEFAULT_SHM, {in.d}, {999}}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {}, {{{}, {}, {h, PAD}, {w, PAD}}}, {out.d}}}},
			{-5, 2});
	});
	dump("filter3x3", 0, out);
}

// ---- main/wfilter3x3.cu:8-15 and :17-69 ----
struct WeightedSum {
	int total;
	struct Constant { int init; };
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = c.init; }
	STRATEGY_LOOP_STUB(2, 0) { total += IMEM(0, 0) * IMEM(1, 0); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total; }
};

void app_wfilter3x3() {
	const int w = 300, h = 250;
	DevBuf<int> in(iota_vec((size_t)w * h)), out((size_t)w * h);
	DevBuf<int> wt(std::vector<int>{1, 2, 1, 2, 4, 2, 1, 2, 1});
	timed("wfilter3x3", 0, [&] {
		return Execute<WeightedSum, 0x111, 0x1122, 0xc0>(
			{{{1, 1, 1, 1}, {1, 1, 1, 1}, {h, 16, 4, 1}, {w, 16, 8, 1}}},
			{{{1, 1}, {1, 1}, {3, 3}, {3, 3}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {{{}, {}, {2, -1, 1}, {3, -1, 1}}},
			   {{{1, PAD}, {1, PAD}, {h, PAD}, {w, PAD}}}, DEFAULT_SHM, {in.d}, {56}},
			  {{{{}, {}, {}, {}}}, {{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {{{1, PAD}, {1, PAD}, {3, PAD}, {3, PAD}}},
			   DEFAULT_SHM, {wt.d}, {}}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {}, {{{}, {}, {h, PAD}, {w, PAD}}}, {out.d}}}},
			{-5});
	});
	dump("wfilter3x3", 0, out);
}

// ---- main/bilateral.cu:9-24 and :26-101 ----
struct RangeWeighted {
	float wsum, wxsum, centre;
	struct Constant { float norm; };
	STRATEGY_TYPEDEF_STUB(float, Constant)
	STRATEGY_PRE_STUB(1, 0) {
		wsum = 0.0f;
		wxsum = 0.0f;
		centre = IMEM(0, 0);
	}
	STRATEGY_LOOP_STUB(3, 0) {
		const float v = IMEM(0, 0), diff = v - centre;
		const float wgt = expf(diff * diff * c.norm) * IMEM(1, 0) * IMEM(2, 0);
		wsum += wgt;
		wxsum += wgt * v;
	}
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = wxsum / wsum; }
};

void app_bilateral() {
	const int w = 300, h = 250;
	const float s1 = 4.0f, s2 = 10.0f;
	const float n1 = -1.0f / (2.0f * s1 * s1), n2 = -1.0f / (2.0f * s2 * s2);
	const int ofs = (int)(s1 * 3.0f), k = 2 * ofs + 1;
	std::vector<float> x((size_t)w * h), ws(k);
	std::iota(x.begin(), x.end(), 0.0f);
	for (int i = 0; i < k; ++i) ws[i] = (float)std::exp((double)((i - ofs) * (i - ofs)) * (double)n1);
	DevBuf<float> in(x), wd(ws), out((size_t)w * h);
	timed("bilateral", 0, [&] {
		return Execute<RangeWeighted, 0x11111>(
			{{{1, 1, 1, 1}, {1, 1, 1, 1}, {h, 16, 2, 1}, {w, 16, 16, 1}}},
			{{{1, 1}, {1, 1}, {k, k}, {k, k}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {{{}, {}, {}, {}}}, {{{1, PAD}, {1, PAD}, {h, PAD}, {w, PAD}}},
			   DEFAULT_SHM, {in.d}, {}},
			  {{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {{{}, {}, {2, -ofs, 1}, {3, -ofs, 1}}},
			   {{{1, PAD}, {1, PAD}, {h, PAD}, {w, PAD}}}, DEFAULT_SHM, {in.d}, {0.0f}},
			  {{{{}, {}, {}, {}}}, {{{}, {}, {3, 0, 1}, {}}}, {{{1, PAD}, {1, PAD}, {1, PAD}, {k, PAD}}}, DEFAULT_SHM,
			   {wd.d}, {}},
			  {{{{}, {}, {}, {}}}, {{{}, {}, {}, {3, 0, 1}}}, {{{1, PAD}, {1, PAD}, {1, PAD}, {k, PAD}}}, DEFAULT_SHM,
			   {wd.d}, {}}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {}, {{{}, {}, {h, PAD}, {w, PAD}}}, {out.d}}}},
			{n2});
	});
	dump("bilateral", 0, out);
}

// ---- main/cost_volume.cu:8-15 and :17-65 ----
struct AbsDiffSum {
	int sad;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { sad = 0; }
	STRATEGY_LOOP_STUB(2, 0) { sad += abs(IMEM(0, 0) - IMEM(1, 0)); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = sad; }
};

void app_cost_volume() {
	const int w = 1920, h = 1080, k = 7, sr = 15, ko = k / 2, so = sr / 2;
	DevBuf<int> f(iota_vec((size_t)w * h)), cv((size_t)w * h * sr);
	timed("cost_volume", 0, [&] {
		return Execute<AbsDiffSum, 0x111>(
			{{{1, 1, 1, 1}, {h, 4, 1, 1}, {w, 8, 2, 1}, {sr, 16, 16, 1}}},
			{{{1, 1}, {1, 1}, {1, 1}, {k, k}}},
			{{{{{{}, {2, 0, 1}, {3, 0, 1}, {3, -so, 1}}}, {{{}, {}, {}, {3, -ko, 1}}},
			   {{{1, WRAP}, {1, WRAP}, {h, WRAP}, {w, WRAP}}}, DEFAULT_SHM, {f.d}, {}},
			  {{{{}, {2, 0, 1}, {3, 0, 1}, {}}}, {{{}, {}, {}, {3, -ko, 1}}},
			   {{{1, WRAP}, {1, WRAP}, {h, WRAP}, {w, WRAP}}}, DEFAULT_SHM, {f.d}, {}}}},
			{{{{{{}, {1, 0, 1}, {2, 0, 1}, {3, 0, 1}}}, {}, {{{1, WRAP}, {h, WRAP}, {w, WRAP}, {sr, WRAP}}}, {cv.d}}}});
	});
	dump("cost_volume", 0, cv);
}

// ---- main/full_me.cu:17-64 (strategy as cost_volume) ----
void app_full_me() {
	const int w = 1920, h = 1080, b = 8, so = -7, sr = 15;
	DevBuf<int> f(iota_vec((size_t)w * h)), sad((size_t)(w / b) * (h / b) * sr * sr);
	timed("full_me", 0, [&] {
		return Execute<AbsDiffSum, 0x111, 0x2211>(
			{{{h / b, 1, 1, 1}, {w / b, 1, 1, 1}, {sr, 16, 2, 1}, {sr, 16, 16, 1}}},
			{{{1, 1}, {1, 1}, {b, b}, {b, b}}},
			{{{{{{2, 0, b}, {3, 0, b}, {2, so, 1}, {3, so, 1}}}, {{{}, {}, {2, 0, 1}, {3, 0, 1}}},
			   {{{1, WRAP}, {1, WRAP}, {h, WRAP}, {w, WRAP}}}, DEFAULT_SHM, {f.d}, {}},
			  {{{{2, 0, b}, {3, 0, b}, {}, {}}}, {{{}, {}, {2, 0, 1}, {3, 0, 1}}},
			   {{{1, WRAP}, {1, WRAP}, {h, WRAP}, {w, WRAP}}}, DEFAULT_SHM, {f.d}, {}}}},
			{{{{{{0, 0, 1}, {1, 0, 1}, {2, 0, 1}, {3, 0, 1}}}, {},
			   {{{h / b, WRAP}, {w / b, WRAP}, {sr, WRAP}, {sr, WRAP}}}, {sad.d}}}});
	});
	dump("full_me", 0, sad);
}

// ---- main/iimg.cu:11-18 and :20-82 (two calls; the second leaves warp_shuf at 0) ----
struct RunningSum {
	int total;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = 0; }
	STRATEGY_LOOP_STUB(1, 1) { OMEM(0, 0) = total += IMEM(0, 0); }
	STRATEGY_POST_STUB_
};

void app_iimg() {
	const int w = 500, h = 300;
	DevBuf<int> in(std::vector<int>((size_t)w * h, 1)), tmp((size_t)w * h), out((size_t)w * h);
	timed("iimg", 0, [&] {
		return Execute<RunningSum, 0x11>(
			{{{1, 1, 1, 1}, {1, 1, 1, 1}, {1, 1, 1, 1}, {h, 128, 32, 1}}},
			{{{1, 1}, {1, 1}, {1, 1}, {w, 32}}},
			{{{{{{}, {}, {}, {2, 0, 1}}}, {{{}, {}, {}, {3, 0, 1}}}, {{{1, PAD}, {1, PAD}, {h, PAD}, {w, PAD}}},
			   DEFAULT_SHM, {in.d}, {}}}},
			{{{{{{}, {}, {}, {3, 0, 1}}}, {{{}, {}, {}, {2, 0, 1}}}, {{{1, PAD}, {1, PAD}, {w, PAD}, {h, PAD}}},
			   {tmp.d}}}},
			{});
	});
	dump("iimg", 0, tmp);
	timed("iimg", 1, [&] {
		return Execute<RunningSum, 0x11>(
			{{{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {w, 128, 32}}},
			{{{1, 1}, {1, 1}, {1, 1}, {h, 32}}},
			{{{{{{}, {}, {}, {2, 0, 1}}}, {{{}, {}, {}, {3, 0, 1}}}, {{{1, PAD}, {1, PAD}, {w, PAD}, {h, PAD}}}, {},
			   {tmp.d}, {}}}},
			{{{{{{}, {}, {}, {3, 0, 1}}}, {{{}, {}, {}, {2, 0, 1}}}, {{{1, PAD}, {1, PAD}, {h, PAD}, {w, PAD}}},
			   {out.d}}}},
			{});
	});
	dump("iimg", 1, out);
}

// ---- main/gemm.cu:8-15 and :17-67 ----
struct Dot {
	int total;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = 0; }
	STRATEGY_LOOP_STUB(2, 0) { total += IMEM(0, 0) * IMEM(1, 0); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total; }
};

void app_gemm() {
	const int m = 100, k = 100, n = 200;
	DevBuf<int> A(iota_vec((size_t)m * k)), B(iota_vec((size_t)k * n)), C((size_t)m * n);
	timed("gemm", 0, [&] {
		return Execute<Dot, 0x111, 0x1124, 0x48>(
			{{{1, 1, 1, 1}, {1, 1, 1, 1}, {m, 16, 2, 1}, {n, 16, 16, 1}}},
			{{{1, 1}, {1, 1}, {1, 1}, {k, 16}}},
			{{{{{{}, {}, {2, 0, 1}, {}}}, {{{}, {}, {}, {3, 0, 1}}}, {{{1, PAD}, {1, PAD}, {m, PAD}, {k, PAD}}},
			   DEFAULT_SHM, {A.d}, {}},
			  {{{{}, {}, {}, {3, 0, 1}}}, {{{}, {}, {}, {2, 0, 1}}}, {{{1, PAD}, {1, PAD}, {k, PAD}, {n, PAD}}},
			   DEFAULT_SHM, {B.d}, {}}}},
			{{{{{{}, {}, {2, 0, 1}, {3, 0, 1}}}, {}, {{{}, {}, {m, PAD}, {n, PAD}}}, {C.d}}}});
	});
	dump("gemm", 0, C);
}

// ---- main/fprop.cu:10-17 and :19-82 ----
void app_fprop() {
	const int iw = 80, ih = 64, f = 7, ofs = -f / 2, s = 2, ich = 40, och = 60, ow = iw / s, oh = ih / s, bs = 32;
	std::vector<int> x((size_t)iw * ih * ich * bs), wt((size_t)och * ich * f * f);
	std::default_random_engine gen;
	std::uniform_int_distribution<int> dist(0, 10);
	for (auto& v : x) v = dist(gen);
	for (auto& v : wt) v = dist(gen);
	DevBuf<int> in(x), wd(wt), out((size_t)ow * oh * och * bs);
	timed("fprop", 0, [&] {
		return Execute<Dot>(
			{{{bs, 1, 1, 1}, {och, 4, 1, 1}, {oh, 8, 4, 1}, {ow, 8, 8, 1}}},
			{{{1, 1}, {ich, 6}, {f, f}, {f, f}}},
			{{{{{{0, 0, 1}, {}, {2, 0, s}, {3, 0, s}}}, {{{}, {1, 0, 1}, {2, ofs, 1}, {3, ofs, 1}}},
			   {{{bs, PAD}, {ich, PAD}, {ih, PAD}, {iw, PAD}}}, DEFAULT_SHM, {in.d}, {}},
			  {{{{}, {0, 0, 1}, {}, {}}}, {{{}, {1, 0, 1}, {2, 0, 1}, {3, 0, 1}}},
			   {{{och, PAD}, {ich, PAD}, {f, PAD}, {f, PAD}}}, DEFAULT_SHM, {wd.d}, {}}}},
			{{{{{{0, 0, 1}, {1, 0, 1}, {2, 0, 1}, {3, 0, 1}}}, {}, {{{bs, PAD}, {och, PAD}, {oh, PAD}, {ow, PAD}}},
			   {out.d}}}});
	});
	dump("fprop", 0, out);
}

}  // namespace

int main(int argc, char** argv) {
	if (argc < 2) {
		std::fprintf(stderr, "usage: %s <outdir> [app]\n", argv[0]);
		return 2;
	}
	g_dir = argv[1];
	const std::string only = argc > 2 ? argv[2] : "";
	struct { const char* name; void (*fn)(); } apps[] = {
		{"filter3x3", app_filter3x3}, {"wfilter3x3", app_wfilter3x3}, {"bilateral", app_bilateral},
		{"cost_volume", app_cost_volume}, {"full_me", app_full_me}, {"iimg", app_iimg},
		{"gemm", app_gemm}, {"fprop", app_fprop},
	};
	for (auto& a : apps)
		if (only.empty() || only == a.name) a.fn();
	return g_fail ? 1 : 0;
}
