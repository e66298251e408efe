/* C restatement of the reference optimizer's per-frequency algorithm
 * (pngf-opt/pngfopt.hpp, pngf-opt/linalg.hpp) on C^-1.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle at full sizes and the timed CPU
 * baseline. LAPACK/BLAS routines are supplied at run time as function
 * pointers (the Python side takes them from scipy's bundled OpenBLAS), as the
 * reference links OpenBLAS (pngf-opt/Makefile:28).
 */
#ifndef PNGF_PORT_H
#define PNGF_PORT_H

typedef struct port_state port_state;

void port_set_lapack(void *zgetrf, void *zgetri, void *zgetrs, void *zgemm);

/* G: n x n complex128 column-major; Gobj: E x n column-major (row 0 built
 * from the port by the caller); Einc: n; P: n 0/1. Builds C, inverts it
 * (zgetrf + zgetri), PEinc, R, S, Eobj (pngfopt.hpp:196-250, 542-552;
 * linalg.hpp:34-85). Returns NULL on failure. */
port_state *port_create(long n, int E, int kmax, const double *G, const double *Gobj, const double *Einc,
                        const signed char *P);
void port_destroy(port_state *s);
/* compute_updated_Eobj for the flip set (s, d) (pngfopt.hpp:379-539). */
int port_eval(port_state *s, const int *edges, const int *signs, int k, double *new_eobj);
/* update_C_inv + compute_PEinc + compute_R_matrix(0) (pngfopt.hpp:256-367, 542-552, 237-250). */
int port_accept(port_state *s);
void port_eobj(const port_state *s, double *eobj);
int port_threads(void);

#endif
