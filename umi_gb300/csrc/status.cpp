// Status codes and per-thread error detail.
#include <cstdio>
#include <cstring>

#include "common.h"

namespace {
thread_local char g_detail[512] = "";
}

namespace umi {

umi_status fail(umi_status st, const char* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	std::vsnprintf(g_detail, sizeof(g_detail), fmt, ap);
	va_end(ap);
	return st;
}

umi_status ok() {
	g_detail[0] = '\0';
	return UMI_OK;
}

umi_status cuda_status(cudaError_t e, const char* what) {
	if (e == cudaSuccess) return UMI_OK;
	return fail(UMI_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

}  // namespace umi

extern "C" const char* umi_status_string(int status) {
	switch (status) {
		case UMI_OK: return "UMI_OK";
		case UMI_ERR_INVALID_DESC: return "UMI_ERR_INVALID_DESC";
		case UMI_ERR_INVALID_ARG: return "UMI_ERR_INVALID_ARG";
		case UMI_ERR_UNSUPPORTED: return "UMI_ERR_UNSUPPORTED";
		case UMI_ERR_CUDA: return "UMI_ERR_CUDA";
		case UMI_ERR_NO_MEMORY: return "UMI_ERR_NO_MEMORY";
		case UMI_ERR_TIMEOUT: return "UMI_ERR_TIMEOUT";
		default: return "UMI_ERR_UNKNOWN";
	}
}

extern "C" const char* umi_last_error_string(void) { return g_detail; }

extern "C" int umi_version(void) { return 100; }
