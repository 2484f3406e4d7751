// Host/device mirror buffers with the interface of the reference's
// src/SyncedMemory.h (MemoryBuffer<T>, SyncedMemory<T> and their
// get_{cpu,gpu}_{ro,wo,rw} accessors), so that applications written against
// the reference compile unchanged.  Differences: buffers are released
// (the reference's MemoryBuffer::Free tests the wrong pointer, leaking every
// buffer, src/SyncedMemory.h:72), moves keep the size and state, and CUDA
// failures are reported on stderr instead of being ignored.
#pragma once
#include <cuda_runtime.h>

#include <cassert>
#include <cstddef>
#include <cstdio>

namespace umi_compat {
inline void report(cudaError_t e, const char* what) {
	if (e != cudaSuccess) std::fprintf(stderr, "SyncedMemory: %s: %s\n", what, cudaGetErrorString(e));
}
}  // namespace umi_compat

template <typename T>
class SyncedMemory {
	enum MemoryState { GPU_IS_NEW, CPU_IS_NEW, SYNCED } state_ = SYNCED;
	T *cpu_ = nullptr, *gpu_ = nullptr;
	size_t n_ = 0;

	void Sync() {
		if (state_ == CPU_IS_NEW)
			umi_compat::report(cudaMemcpy(gpu_, cpu_, sizeof(T) * n_, cudaMemcpyHostToDevice), "host to device");
		else if (state_ == GPU_IS_NEW)
			umi_compat::report(cudaMemcpy(cpu_, gpu_, sizeof(T) * n_, cudaMemcpyDeviceToHost), "device to host");
		state_ = SYNCED;
	}

public:
	SyncedMemory() {}
	SyncedMemory(T* cpu, T* gpu, size_t n) : cpu_(cpu), gpu_(gpu), n_(n) {}
	void Reset(T* cpu, T* gpu, size_t n) { cpu_ = cpu; gpu_ = gpu; n_ = n; state_ = SYNCED; }
	SyncedMemory(const SyncedMemory&) = delete;
	SyncedMemory& operator=(const SyncedMemory&) = delete;
	SyncedMemory(SyncedMemory&& m) : state_(m.state_), cpu_(m.cpu_), gpu_(m.gpu_), n_(m.n_) { m.cpu_ = m.gpu_ = nullptr; }
	SyncedMemory& operator=(SyncedMemory&& m) {
		if (this != &m) {
			state_ = m.state_; cpu_ = m.cpu_; gpu_ = m.gpu_; n_ = m.n_;
			m.cpu_ = m.gpu_ = nullptr;
		}
		return *this;
	}
	T* get_cpu_wo() { state_ = CPU_IS_NEW; return cpu_; }
	T* get_gpu_wo() { state_ = GPU_IS_NEW; return gpu_; }
	const T* get_cpu_ro() { if (state_ != CPU_IS_NEW) Sync(); return cpu_; }
	const T* get_gpu_ro() { if (state_ != GPU_IS_NEW) Sync(); return gpu_; }
	T* get_cpu_rw() { get_cpu_ro(); return get_cpu_wo(); }
	T* get_gpu_rw() { get_gpu_ro(); return get_gpu_wo(); }
};

template <typename T>
class MemoryBuffer {
	T *cpu_ = nullptr, *gpu_ = nullptr;
	void Alloc(size_t n) {
		if (n == 0) return;
		cpu_ = new T[n];
		umi_compat::report(cudaMalloc(&gpu_, sizeof(T) * n), "cudaMalloc");
	}

public:
	void Free() {
		delete[] cpu_;
		if (gpu_) umi_compat::report(cudaFree(gpu_), "cudaFree");
		cpu_ = gpu_ = nullptr;
	}
	void Realloc(size_t n) { Free(); Alloc(n); }
	MemoryBuffer(size_t n = 0) { Alloc(n); }
	~MemoryBuffer() { Free(); }
	MemoryBuffer(const MemoryBuffer&) = delete;
	MemoryBuffer& operator=(const MemoryBuffer&) = delete;
	MemoryBuffer(MemoryBuffer&& b) : cpu_(b.cpu_), gpu_(b.gpu_) { b.cpu_ = b.gpu_ = nullptr; }
	MemoryBuffer& operator=(MemoryBuffer&& b) {
		if (this != &b) { Free(); cpu_ = b.cpu_; gpu_ = b.gpu_; b.cpu_ = b.gpu_ = nullptr; }
		return *this;
	}
	SyncedMemory<T> CreateSync(size_t n, size_t offset = 0) { return SyncedMemory<T>(cpu_ + offset, gpu_ + offset, n); }
};
