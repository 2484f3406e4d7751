// Randomised-descriptor check of the generic GPU path (UMI::Execute in
// include/umi/UMI_gpu.h) against the CPU oracle interpreter
// (oracle/umi_interp.hpp), on the same descriptors and inputs.
//
// Each trial draws parallel / accumulation spaces, tilings (valid per the
// reference's rules), Expand words, view maps (offsets, negative strides,
// several view dimensions folded onto one physical dimension, offsets 2^30
// outside the extent that take the 64-bit index path), physical
// sizes and PAD/WRAP modes, then runs three strategies that exercise every
// stage and memory kind: multi-pointer Loop inputs with several Post outputs,
// Pre and Post inputs and outputs, and Loop outputs (a running sum).  Integer
// results must match exactly, including untouched output elements.  Invalid
// descriptors must be rejected by both.
//
// Usage: generic_fuzz [trials] [seed]   (prints one JSON summary line)
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "umi/UMI_gpu.h"
#include "../../oracle/umi_interp.hpp"

using namespace UMI;

namespace {

struct Rng {
	uint64_t s;
	uint32_t next() {
		s = s * 6364136223846793005ull + 1442695040888963407ull;
		return (uint32_t)(s >> 33);
	}
	int uni(int lo, int hi) { return lo + (int)(next() % (uint32_t)(hi - lo + 1)); }
};

// Loop input with two pointers, two Post outputs.
struct TwoPtr {
	int acc;
	struct Constant { int init; };
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { acc = c.init; }
	STRATEGY_LOOP_STUB(1, 0) { acc = acc * 3 + IMEM(0, 0) - 2 * IMEM(0, 1); }
	STRATEGY_POST_STUB(0, 2) {
		OMEM(0, 0) = acc;
		OMEM(1, 0) = acc ^ 0x55;
	}
};
// Pre and Post memories.
struct Stages {
	int acc, first;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(1, 1) {
		first = IMEM(0, 0);
		acc = 2 * first;
		OMEM(0, 0) = first + 1;
	}
	STRATEGY_LOOP_STUB(2, 0) { acc += IMEM(0, 0) * IMEM(1, 0) + 1; }
	STRATEGY_POST_STUB(1, 1) { OMEM(0, 0) = acc - 7 * IMEM(0, 0) + first; }
};
// Loop output: running sum written at (p, a).
struct Scan {
	int acc;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { acc = 0; }
	STRATEGY_LOOP_STUB(1, 1) { OMEM(0, 0) = acc += IMEM(0, 0); }
	STRATEGY_POST_STUB_
};

struct Phys {
	NDTuple<PhysicalDim> dims;
	size_t n() const {
		size_t v = 1;
		for (auto& d : dims) v *= (size_t)d.size;
		return v;
	}
};

NDTuple<ParallelDim> rand_pdims(Rng& r, const int (&tot)[4]) {
	int wexp[4] = {0, 0, 0, 0};
	for (int i = 0; i < 5; ++i) ++wexp[r.uni(0, 3)];
	NDTuple<ParallelDim> p;
	int threads = 1;
	for (int d = 0; d < 4; ++d) {
		const int w = 1 << wexp[d];
		const int shuf = r.uni(0, 3) == 0 ? 2 : (r.uni(0, 1) ? 1 : 0);  // 0 reads as 1
		const int sh = shuf == 0 ? 1 : shuf;
		int blk = w * sh;
		if (threads * blk * 2 <= 256 && r.uni(0, 3) == 0) blk *= 2;
		threads *= blk;
		p[d] = ParallelDim{tot[d], blk, w, shuf};
	}
	if (threads > 1024)  // keep within one CTA: fall back to one warp per CTA
		for (int d = 0; d < 4; ++d) p[d] = ParallelDim{tot[d], p[d].warp_size, p[d].warp_size, 1};
	return p;
}

Phys rand_phys(Rng& r) {
	Phys ph;
	for (int k = 0; k < 4; ++k)
		ph.dims[k] = PhysicalDim{r.uni(1, 6), r.uni(0, 1) ? PhysicalDim::PAD : PhysicalDim::WRAP};
	return ph;
}

NDTuple<ViewDim> rand_view(Rng& r, bool active) {
	NDTuple<ViewDim> v;
	for (int d = 0; d < 4; ++d)
		v[d] = active ? ViewDim{r.uni(0, 3), r.uni(-2, 2), r.uni(-1, 2)} : ViewDim{0, 0, 0};
	return v;
}

std::vector<int> rand_data(Rng& r, size_t n) {
	std::vector<int> v(n);
	for (auto& x : v) x = r.uni(-50, 50);
	return v;
}

template <class T>
T* upload(const std::vector<T>& h) {
	T* d = nullptr;
	cudaMalloc(&d, h.size() * sizeof(T) + 16);
	cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
	return d;
}

template <class T>
std::vector<T> download(const T* d, size_t n) {
	std::vector<T> h(n);
	cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
	return h;
}

int g_trials = 0, g_fail = 0, g_rejected_ok = 0;

// Output physical dims shaped like P (identity view): every point writes its own element.
NDTuple<PhysicalDim> p_shaped(const int (&tot)[4]) {
	NDTuple<PhysicalDim> o;
	for (int d = 0; d < 4; ++d) o[d] = PhysicalDim{tot[d], PhysicalDim::PAD};
	return o;
}
NDTuple<ViewDim> identity_view() { return {{{0, 0, 1}, {1, 0, 1}, {2, 0, 1}, {3, 0, 1}}}; }

template <uint64_t E>
void trial_twoptr(Rng& r) {
	int tot[4];
	for (int d = 0; d < 4; ++d) tot[d] = r.uni(1, 4);
	const auto pd = rand_pdims(r, tot);
	NDTuple<AccumulationDim> ad;
	for (int d = 0; d < 4; ++d) ad[d] = AccumulationDim{r.uni(0, 3) == 0 ? 1 : r.uni(1, 3), r.uni(1, 3)};
	Phys ph = rand_phys(r);
	auto d0 = rand_data(r, ph.n()), d1 = rand_data(r, ph.n());
	int *g0 = upload(d0), *g1 = upload(d1);
	const size_t no = (size_t)tot[0] * tot[1] * tot[2] * tot[3];
	std::vector<int> init(no, -12345);
	int *o0 = upload(init), *o1 = upload(init);
	std::vector<int> c0 = init, c1 = init;
	const int pv = r.uni(-9, 9), pw = r.uni(-9, 9);
	UnrolledI<int> im{rand_view(r, true), rand_view(r, true), ph.dims, DEFAULT_SHM, {g0, g1}, {pv, pw}};
	if (r.uni(0, 3) == 0) {
		// a view offset 2^30 outside the extent: every coordinate on that physical
		// dimension clamps, and the call no longer fits 32-bit indices, so the
		// launch takes the 64-bit instantiation of the kernel
		const int d = r.uni(0, 3);
		im.p_view_dims[d].ofs += r.uni(0, 1) ? (1 << 30) : -(1 << 30);
	}
	UnrolledI<int> imc{im.p_view_dims, im.a_view_dims, ph.dims, DEFAULT_SHM, {d0.data(), d1.data()}, {pv, pw}};
	UnrolledO<int> om0{identity_view(), rand_view(r, false), p_shaped(tot), {o0}};
	UnrolledO<int> om1{identity_view(), rand_view(r, false), p_shaped(tot), {o1}};
	UnrolledO<int> cm0{identity_view(), om0.a_view_dims, p_shaped(tot), {c0.data()}};
	UnrolledO<int> cm1{identity_view(), om1.a_view_dims, p_shaped(tot), {c1.data()}};
	const int init_c = r.uni(-5, 5);
	const umi_status st = Execute<TwoPtr, 0x112, E>(pd, ad, {{im}}, {{om0, om1}}, {init_c});
	const int rc = umi_oracle::Interpret<TwoPtr, 0x112, E>(pd, ad, {{imc}}, {{cm0, cm1}}, {init_c});
	cudaDeviceSynchronize();
	++g_trials;
	if ((st == UMI_OK) != (rc == 0)) { ++g_fail; std::fprintf(stderr, "twoptr: status %d vs oracle %d\n", st, rc); }
	else if (st == UMI_OK) {
		if (download(o0, no) != c0 || download(o1, no) != c1) { ++g_fail; std::fprintf(stderr, "twoptr mismatch\n"); }
	} else ++g_rejected_ok;
	cudaFree(g0); cudaFree(g1); cudaFree(o0); cudaFree(o1);
}

template <uint64_t E>
void trial_stages(Rng& r) {
	int tot[4];
	for (int d = 0; d < 4; ++d) tot[d] = r.uni(1, 4);
	const auto pd = rand_pdims(r, tot);
	NDTuple<AccumulationDim> ad;
	for (int d = 0; d < 4; ++d) ad[d] = AccumulationDim{r.uni(1, 3), r.uni(1, 2)};
	Phys pa = rand_phys(r), pb = rand_phys(r), pc = rand_phys(r), pe = rand_phys(r);
	auto da = rand_data(r, pa.n()), db = rand_data(r, pb.n()), dc = rand_data(r, pc.n()), de = rand_data(r, pe.n());
	int *ga = upload(da), *gb = upload(db), *gc = upload(dc), *ge = upload(de);
	const size_t no = (size_t)tot[0] * tot[1] * tot[2] * tot[3];
	std::vector<int> init(no, 777);
	int *o0 = upload(init), *o1 = upload(init);
	std::vector<int> c0 = init, c1 = init;
	UnrolledI<int> i0{rand_view(r, true), rand_view(r, true), pa.dims, DEFAULT_SHM, {ga}, {3}};
	UnrolledI<int> i1{rand_view(r, true), rand_view(r, true), pb.dims, DEFAULT_SHM, {gb}, {-4}};
	UnrolledI<int> i2{rand_view(r, true), rand_view(r, true), pc.dims, DEFAULT_SHM, {gc}, {5}};
	UnrolledI<int> i3{rand_view(r, true), rand_view(r, true), pe.dims, DEFAULT_SHM, {ge}, {6}};
	UnrolledI<int> j0{i0.p_view_dims, i0.a_view_dims, pa.dims, DEFAULT_SHM, {da.data()}, {3}};
	UnrolledI<int> j1{i1.p_view_dims, i1.a_view_dims, pb.dims, DEFAULT_SHM, {db.data()}, {-4}};
	UnrolledI<int> j2{i2.p_view_dims, i2.a_view_dims, pc.dims, DEFAULT_SHM, {dc.data()}, {5}};
	UnrolledI<int> j3{i3.p_view_dims, i3.a_view_dims, pe.dims, DEFAULT_SHM, {de.data()}, {6}};
	UnrolledO<int> om0{identity_view(), {}, p_shaped(tot), {o0}}, om1{identity_view(), {}, p_shaped(tot), {o1}};
	UnrolledO<int> cm0{identity_view(), {}, p_shaped(tot), {c0.data()}}, cm1{identity_view(), {}, p_shaped(tot), {c1.data()}};
	const umi_status st = Execute<Stages, 0x1111111111111111ull, E>(pd, ad, {{i0, i1, i2, i3}}, {{om0, om1}});
	const int rc = umi_oracle::Interpret<Stages, 0x1111111111111111ull, E>(pd, ad, {{j0, j1, j2, j3}}, {{cm0, cm1}});
	cudaDeviceSynchronize();
	++g_trials;
	if ((st == UMI_OK) != (rc == 0)) { ++g_fail; std::fprintf(stderr, "stages: status %d vs oracle %d\n", st, rc); }
	else if (st == UMI_OK) {
		if (download(o0, no) != c0 || download(o1, no) != c1) { ++g_fail; std::fprintf(stderr, "stages mismatch\n"); }
	} else ++g_rejected_ok;
	cudaFree(ga); cudaFree(gb); cudaFree(gc); cudaFree(ge); cudaFree(o0); cudaFree(o1);
}

template <uint64_t E>
void trial_scan(Rng& r) {
	// P on dims 2,3 and A on dims 2,3 so that (p, a) -> output element is injective.
	int tot[4] = {1, 1, r.uni(1, 6), r.uni(1, 6)};
	const auto pd = rand_pdims(r, tot);
	NDTuple<AccumulationDim> ad{{{1, 1}, {1, 1}, {r.uni(1, 5), r.uni(1, 3)}, {r.uni(1, 5), r.uni(1, 3)}}};
	Phys ph = rand_phys(r);
	auto di = rand_data(r, ph.n());
	int* gi = upload(di);
	NDTuple<PhysicalDim> op{{{tot[2], PhysicalDim::PAD}, {tot[3], PhysicalDim::PAD},
	                         {ad[2].total_size, PhysicalDim::PAD}, {ad[3].total_size, PhysicalDim::PAD}}};
	const size_t no = (size_t)tot[2] * tot[3] * ad[2].total_size * ad[3].total_size;
	std::vector<int> init(no, 31337);
	int* o = upload(init);
	std::vector<int> co = init;
	UnrolledI<int> im{rand_view(r, true), rand_view(r, true), ph.dims, DEFAULT_SHM, {gi}, {11}};
	UnrolledI<int> imc{im.p_view_dims, im.a_view_dims, ph.dims, DEFAULT_SHM, {di.data()}, {11}};
	const NDTuple<ViewDim> opv{{{}, {}, {0, 0, 1}, {1, 0, 1}}}, oav{{{}, {}, {2, 0, 1}, {3, 0, 1}}};
	UnrolledO<int> om{opv, oav, op, {o}};
	UnrolledO<int> cm{opv, oav, op, {co.data()}};
	const umi_status st = Execute<Scan, 0x11, E>(pd, ad, {{im}}, {{om}});
	const int rc = umi_oracle::Interpret<Scan, 0x11, E>(pd, ad, {{imc}}, {{cm}});
	cudaDeviceSynchronize();
	++g_trials;
	if ((st == UMI_OK) != (rc == 0)) { ++g_fail; std::fprintf(stderr, "scan: status %d vs oracle %d\n", st, rc); }
	else if (st == UMI_OK) {
		if (download(o, no) != co) { ++g_fail; std::fprintf(stderr, "scan mismatch\n"); }
	} else ++g_rejected_ok;
	cudaFree(gi); cudaFree(o);
}

void trial_invalid(Rng& r) {
	int tot[4] = {2, 2, 2, 2};
	auto pd = rand_pdims(r, tot);
	switch (r.uni(0, 2)) {
		case 0: pd[3].warp_shuf = 3; break;                 // not a power of two
		case 1: pd[3].warp_size *= 2; break;                // product of warps != 32
		default: {  // block not divisible by warp*shuf (pick the dim with the widest warp, >= 2)
			int d = 0;
			for (int i = 1; i < 4; ++i)
				if (pd[i].warp_size > pd[d].warp_size) d = i;
			pd[d].block_size = pd[d].warp_size * (pd[d].warp_shuf ? pd[d].warp_shuf : 1) + 1;
			break;
		}
	}
	NDTuple<AccumulationDim> ad{{{1, 1}, {1, 1}, {2, 1}, {2, 1}}};
	std::vector<int> d(16, 1);
	int* g = upload(d);
	std::vector<int> c(16, 0);
	int* o = upload(c);
	const NDTuple<PhysicalDim> ph{{{2, PhysicalDim::PAD}, {2, PhysicalDim::PAD}, {2, PhysicalDim::PAD}, {2, PhysicalDim::PAD}}};
	UnrolledI<int> im{identity_view(), {}, ph, DEFAULT_SHM, {g}, {0}};
	UnrolledI<int> imc{identity_view(), {}, ph, DEFAULT_SHM, {d.data()}, {0}};
	UnrolledO<int> om{identity_view(), {}, ph, {o}}, cm{identity_view(), {}, ph, {c.data()}};
	UnrolledO<int> om2{identity_view(), {}, ph, {o}}, cm2{identity_view(), {}, ph, {c.data()}};
	const umi_status st = Execute<TwoPtr, 0x111>(pd, ad, {{im}}, {{om, om2}}, {0});
	const int rc = umi_oracle::Interpret<TwoPtr, 0x111>(pd, ad, {{imc}}, {{cm, cm2}}, {0});
	++g_trials;
	if (st != UMI_ERR_INVALID_DESC || rc == 0) { ++g_fail; std::fprintf(stderr, "invalid accepted: %d %d\n", st, rc); }
	else ++g_rejected_ok;
	cudaFree(g); cudaFree(o);
}

}  // namespace

int main(int argc, char** argv) {
	const int trials = argc > 1 ? std::atoi(argv[1]) : 200;
	Rng r{argc > 2 ? (uint64_t)std::atoll(argv[2]) : 12345ull};
	for (int t = 0; t < trials; ++t) {
		switch (t % 7) {
			case 0: trial_twoptr<0x1111>(r); break;
			case 1: trial_twoptr<0x2112>(r); break;
			case 2: trial_stages<0x1111>(r); break;
			case 3: trial_stages<0x1221>(r); break;
			case 4: trial_scan<0x1111>(r); break;
			case 5: trial_scan<0x1123>(r); break;
			default: trial_invalid(r); break;
		}
	}
	const cudaError_t e = cudaDeviceSynchronize();
	std::printf("{\"trials\": %d, \"failures\": %d, \"rejected_as_expected\": %d, \"cuda\": \"%s\"}\n", g_trials, g_fail,
	            g_rejected_ok, cudaGetErrorName(e));
	return (g_fail || e != cudaSuccess) ? 1 : 0;
}
