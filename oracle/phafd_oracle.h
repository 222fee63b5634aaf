/* phafd_oracle.h -- C ABI of the FP64 CPU oracle (test infrastructure only).
 * Shares the enums and parameter structs of include/phafd_gpu.h so that the
 * tests can drive the oracle and the GPU library with the same call sequence. */
#ifndef PHAFD_ORACLE_H
#define PHAFD_ORACLE_H
#include "../include/phafd_gpu.h"
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct oracle_ctx oracle_ctx;
/* chain model shared by the oracle and (as device code) the GPU library */
void oracle_chain_force(const double* u, int n, int b, double kbond, double b0, double kappa,
                        double* f_out, double* tangent_out);
void oracle_chain_displacement(const double* fchain, const double* fpair, const double* t,
                               const double* xi, double dt, double zeta_para, double zeta_perp,
                               double temp, double* disp);
void oracle_bead_gauss(uint32_t seed, uint64_t step, int half, int bead, double* xi3);
#ifdef __cplusplus
}
#endif
#endif
