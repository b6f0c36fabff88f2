/* TEST INFRASTRUCTURE -- not part of the shipped library.
 *
 * CPU restatement of the reference Legendre<->Chebyshev fast multipole
 * transform (spectralDNS/Legendre-to-Chebyshev, src/C/leg2cheb.c and
 * src/C/lambda.c).  Used only as the checker by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  Every function
 * cites the reference lines it restates.  Symbols carry an "orc_" prefix so the
 * oracle can live in one process beside the library under test.
 *
 * Pinning: tests/test_oracle.py checks this port against golden vectors made by
 * running the unmodified reference (tests/golden/make_golden.py) and against the
 * reference's own known-answer values (src/bin/l2c.c:69-74, 695-707). */
#ifndef L2C_ORACLE_H
#define L2C_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_L2C = 0, ORC_C2L = 1, ORC_BOTH = 2 };

typedef struct orc_plan orc_plan;

/* Lambda(z) = Gamma(z+1/2)/Gamma(z+1), lambda.c:65-98 */
double orc_Lambda(double z);
/* Lambda at integer argument (table for z < 256), lambda.c:101-191 */
double orc_LambdaI(size_t z);

/* Plan for one transform length, leg2cheb.c:820-1234 (modal form, M = 18).
 * direction: ORC_L2C, ORC_C2L or ORC_BOTH. */
orc_plan *orc_create(size_t N, size_t maxs, size_t direction);
/* Same with the form: lagrange = 0 modal, 1 nodal (leg2cheb.c:997-1031,
 * 1076-1100; the far-field blocks are then the kernel samples, not their DCT). */
orc_plan *orc_create_ex(size_t N, size_t maxs, size_t direction, size_t lagrange);
void orc_free(orc_plan *p);

/* One transform, leg2cheb.c:1299-1500 (FMM) or leg2cheb.c:152-234 (direct, L < 1).
 * Returns the reference's flop count, 0 when the direction was not planned. */
size_t orc_execute(const double *in, double *out, orc_plan *p, size_t direction,
                   size_t stride);

/* count transforms of one plan, vector v at in + v*dist, out + v*dist, one
 * vector per OpenMP thread (CPU harness for batched workloads). */
size_t orc_execute_batch(const double *in, double *out, orc_plan *p, size_t direction,
                         size_t count, size_t dist, size_t stride);

/* Ragged list: vector v of plans[v]'s length at in + off[v], out + off[v],
 * one vector per OpenMP thread (CPU harness for ragged workloads). */
size_t orc_execute_ragged(const double *in, double *out, orc_plan **plans, const size_t *off,
                          size_t count, size_t direction);

/* Near field only, with the final scaling: directM (leg2cheb.c:236-376, L2C,
 * strided input and output) and directL (leg2cheb.c:378-535, C2L, input is the
 * premultiplied contiguous copy v, output strided).  FMM plans only. */
size_t orc_directM(const double *in, double *out, orc_plan *p, size_t stride);
size_t orc_directL(const double *v, double *out, orc_plan *p, size_t stride);

/* Plan geometry: info[0..5] = N, L, s, Nn, number of blocks N_b, M. */
void orc_plan_info(const orc_plan *p, size_t *info);
/* Plan data, for comparing plan construction (NULL when absent). */
const double *orc_plan_A(const orc_plan *p, size_t direction); /* 3*N_b*M*M */
const double *orc_plan_T(const orc_plan *p);                   /* 2*s*M     */
const double *orc_plan_lambda(const orc_plan *p);              /* a[0..N)   */
const double *orc_plan_B(const orc_plan *p);  /* 171 (modal) or B0 | B1, 2*M*M (nodal) */
const double *orc_plan_BT(const orc_plan *p); /* 171 (modal), NULL (nodal)            */

void orc_set_threads(int n);
/* 1 when built against OpenBLAS (steps 1 and 5 through CBLAS dgemm, as the reference). */
int orc_uses_blas(void);

#ifdef __cplusplus
}
#endif
#endif
