// Shared helpers for the umi_gb300 library (host side + small device utils).
#pragma once
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdint>

#include "umi_gb300.h"

namespace umi {

// Records a failure detail for umi_last_error_string() (thread-local) and
// returns `st`, so call sites can `return fail(UMI_ERR_..., "...")`.
umi_status fail(umi_status st, const char* fmt, ...);
// Clears the thread's error detail and returns UMI_OK.
umi_status ok();
// Maps the result of a CUDA runtime call to a status.
umi_status cuda_status(cudaError_t e, const char* what);
// Checks the launch that was just issued (cudaGetLastError).
inline umi_status launch_status(const char* what) { return cuda_status(cudaGetLastError(), what); }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

template <class T> constexpr T ceil_div(T a, T b) { return (a + b - 1) / b; }

inline bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace umi

#define UMI_TRY(expr)                               \
	do {                                            \
		umi_status _st = (expr);                    \
		if (_st != UMI_OK) return _st;              \
	} while (0)
