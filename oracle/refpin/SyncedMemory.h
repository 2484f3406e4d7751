// Oracle pinning shim for the reference's host/device mirror buffer
// (johnjohnlin/UMI src/SyncedMemory.h).  Both the "cpu" and the "gpu" side
// live in host memory here, because the oracle runs the operator on the CPU.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cassert>
#include <cstddef>
#include <cstring>

template <typename T>
class SyncedMemory {
	enum State { GPU_IS_NEW, CPU_IS_NEW, SYNCED } state_ = SYNCED;
	T *cpu_ = nullptr, *gpu_ = nullptr;
	size_t n_ = 0;
	void Sync() {
		if (state_ == CPU_IS_NEW) std::memcpy(gpu_, cpu_, sizeof(T) * n_);
		if (state_ == GPU_IS_NEW) std::memcpy(cpu_, gpu_, sizeof(T) * n_);
		state_ = SYNCED;
	}
public:
	SyncedMemory() {}
	SyncedMemory(T* cpu, T* gpu, size_t n) : cpu_(cpu), gpu_(gpu), n_(n) {}
	SyncedMemory(const SyncedMemory&) = delete;
	SyncedMemory& operator=(const SyncedMemory&) = delete;
	SyncedMemory(SyncedMemory&& m) : state_(m.state_), cpu_(m.cpu_), gpu_(m.gpu_), n_(m.n_) {
		m.cpu_ = m.gpu_ = nullptr;
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
public:
	MemoryBuffer(size_t n = 0) {
		if (n) { cpu_ = new T[n](); gpu_ = new T[n](); }
	}
	~MemoryBuffer() { delete[] cpu_; delete[] gpu_; }
	MemoryBuffer(const MemoryBuffer&) = delete;
	MemoryBuffer& operator=(const MemoryBuffer&) = delete;
	SyncedMemory<T> CreateSync(size_t n, size_t offset = 0) {
		return SyncedMemory<T>(cpu_ + offset, gpu_ + offset, n);
	}
};

// The reference's bilateral example prints the CUDA error state once.
inline int cudaGetLastError() { return 0; }
inline const char* cudaGetErrorString(int) { return "no error (CPU oracle)"; }
