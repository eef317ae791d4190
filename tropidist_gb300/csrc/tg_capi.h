// Internal: the public C-ABI declarations plus library-internal helpers shared across units.
#pragma once
#include "../../include/tropidist_gb300.h"
#include <cuda_runtime.h>
#include <string>

namespace tg {
int set_error(int code, const char *what);
int cuda_check(cudaError_t e, const char *where);
int sm_count();
cudaStream_t cur_stream();
}  // namespace tg
