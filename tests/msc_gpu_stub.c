/* Test-only stand-in for libmsc_gpu.so when the snippet of INTEGRATION.md is compiled
 * and run on a machine without a GPU: the two entry points the snippet calls, served
 * by the CPU oracle (host pointers where the library takes device ones).  It checks
 * the snippets' types, byte layouts and files against the reference; the GPU results
 * themselves are checked against the oracle by the GPU tests. */
#include <stdint.h>
#include <stdlib.h>

#include "../include/msc_gpu.h"
#include "../oracle/msc_oracle.h"

int msc_steepest_lstar_host(const float* f_host, const int64_t dims[3], uint8_t* grad_host) {
	return oracle_grad_3d(f_host, dims[0], dims[1], dims[2], grad_host, 0) == 0 ? MSC_OK : MSC_ERR_CUDA;
}

const char* msc_last_error_string(void) { return ""; }

int msc_ms_graph_3d(const uint8_t* grad, const float* f, const int64_t dims[3], const int build_arcs[3],
                    int64_t node_cap, int64_t* node_cell, float* node_value, uint8_t* node_dim,
                    uint8_t* node_boundary, int64_t arc_cap, int32_t* arc_lower, int32_t* arc_upper,
                    float* arc_persistence, int64_t counts[2], msc_stream_t stream) {
	(void)stream;
	int64_t c[2];
	if (oracle_ms_graph_3d(grad, f, dims[0], dims[1], dims[2], build_arcs, 0, 0, 0, 0, 0, 0, 0, 0, 0, c)) return MSC_ERR_CUDA;
	counts[0] = c[0];
	counts[1] = c[1];
	const int nodes = node_cell && node_value && node_dim && node_boundary && node_cap >= c[0];
	const int arcs = arc_lower && arc_upper && arc_cap >= c[1];
	if (!nodes && !arcs) return MSC_OK;
	int64_t* cell = (int64_t*)malloc(sizeof(int64_t) * (size_t)(c[0] + 1));
	float* val = (float*)malloc(sizeof(float) * (size_t)(c[0] + 1));
	uint8_t* dim = (uint8_t*)malloc((size_t)(c[0] + 1));
	uint8_t* bnd = (uint8_t*)malloc((size_t)(c[0] + 1));
	int32_t* lo = (int32_t*)malloc(sizeof(int32_t) * (size_t)(c[1] + 1));
	int32_t* up = (int32_t*)malloc(sizeof(int32_t) * (size_t)(c[1] + 1));
	float* pe = (float*)malloc(sizeof(float) * (size_t)(c[1] + 1));
	int rc = oracle_ms_graph_3d(grad, f, dims[0], dims[1], dims[2], build_arcs, c[0], cell, val, dim, bnd, c[1], lo, up,
	                            pe, c);
	for (int64_t i = 0; nodes && i < c[0]; i++) {
		node_cell[i] = cell[i];
		node_value[i] = val[i];
		node_dim[i] = dim[i];
		node_boundary[i] = bnd[i];
	}
	for (int64_t i = 0; arcs && i < c[1]; i++) {
		arc_lower[i] = lo[i];
		arc_upper[i] = up[i];
		if (arc_persistence) arc_persistence[i] = pe[i];
	}
	free(cell); free(val); free(dim); free(bnd); free(lo); free(up); free(pe);
	return rc ? MSC_ERR_CUDA : MSC_OK;
}
