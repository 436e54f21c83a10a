/* A plain C11 caller of the engine's C ABI (include/qcs_gpu.h), using only entry points that need no GPU:
 * status strings, the reference's random stream, the argument checks of qcs_create, and the host planning of
 * the fuser and of the gate-pass planner.  Built with gcc and run by tests/test_host.py::test_plain_c_caller. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "qcs_gpu.h"

static void one_qubit(qcs_gate* g, uint32_t q, uint32_t traits, const double m[8]) {
	memset(g, 0, sizeof(*g));
	g->k = 1;
	g->q0 = q;
	g->traits = traits;
	memcpy(g->m, m, 8 * sizeof(double));
}

int main(void) {
	printf("status %s\n", qcs_status_string(QCS_INVALID_ARGUMENT));

	qcs_rng_handle rng = NULL;
	double u[3] = {0, 0, 0};
	if (qcs_rng_create(7, &rng) != QCS_OK || qcs_rng_uniform(rng, u, 3) != QCS_OK) return 1;
	qcs_rng_destroy(rng);
	printf("uniform %.17g %.17g %.17g\n", u[0], u[1], u[2]);

	qcs_handle h = NULL;
	printf("create_zero_qubits %d\n", qcs_create(0, QCS_FP64, &h));

	/* 16 qubits: H on qubits 0-11, then RZ(0.3 + 0.1 q) on qubits 12-15 */
	qcs_gate gates[16];
	const double r = 1.0 / sqrt(2.0);
	const double hm[8] = {r, 0, r, 0, r, 0, -r, 0};
	for (uint32_t q = 0; q < 12; ++q) one_qubit(&gates[q], q, 0, hm);
	for (uint32_t q = 12; q < 16; ++q) {
		const double t = 0.3 + 0.1 * q;
		const double rz[8] = {cos(t / 2), -sin(t / 2), 0, 0, 0, 0, cos(t / 2), sin(t / 2)};
		one_qubit(&gates[q], q, QCS_TRAIT_DIAGONAL, rz);
	}
	uint32_t ops[4] = {0, 0, 0, 0}, factors[4] = {0, 0, 0, 0};
	size_t npasses = 0;
	const int st = qcs_plan_gate_passes(16, QCS_FP64, gates, 16, ops, factors, 4, &npasses);
	printf("plan %d %zu %u %u\n", st, npasses, ops[0], factors[0]);

	uint64_t masks[16];
	uint32_t ngates[16];
	size_t nblocks = 0;
	const int fst = qcs_fusion_plan(16, gates, 16, 4, masks, ngates, 16, &nblocks);
	uint32_t folded = 0;
	for (size_t b = 0; b < nblocks && b < 16; ++b) folded += ngates[b];
	printf("fusion %d %zu %u\n", fst, nblocks, folded);
	return 0;
}
