/* Test-only stand-in for libmsc_gpu.so when the snippet of INTEGRATION.md is compiled
 * and run on a machine without a GPU: the two entry points the snippet calls, served
 * by the CPU oracle.  It checks the snippet's types, byte layout and file writing
 * against the reference; the GPU .grad itself is checked against the oracle by the
 * GPU tests. */
#include <stdint.h>

#include "../include/msc_gpu.h"
#include "../oracle/msc_oracle.h"

int msc_steepest_lstar_host(const float* f_host, const int64_t dims[3], uint8_t* grad_host) {
	return oracle_grad_3d(f_host, dims[0], dims[1], dims[2], grad_host, 0) == 0 ? MSC_OK : MSC_ERR_CUDA;
}

const char* msc_last_error_string(void) { return ""; }
