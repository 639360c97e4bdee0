/*
 * CPU oracle for the finite-difference hot path of PseudoAcousticModeling.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference stencils
 * (cpp/Modeling.cu, cpp/Migration.cu, cpp/inversion.cu, src/utils.py) used
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  The product library never links or calls it.
 *
 * Two precisions are compiled from one body (pam_oracle_impl.h):
 *   og_*_f32 : FP32 with the reference C++ kernels' literal constants and
 *              term order; built with -ffp-contract=off so every operation
 *              rounds once, as written;
 *   og_*_f64 : FP64 with the exact rational coefficients (src/utils.py:398-402).
 *
 * Pinned against golden vectors produced by running the reference's own
 * Python CPU kernels (src/utils.py) on small grids: tests/golden/.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

/* ---------------- FP32: reference C++ literals (cpp/Modeling.cu:500-504, 560-563) */
#define R float
#define SFX(n) n##_f32
#define FABS fabsf
#define COS cosf
#define SIN sinf
#define C0 (-2.847222222222f)
#define C1 (1.6f)
#define C2 (-0.2f)
#define C3 (0.02539682539f)
#define C4 (-0.00178571428f)
#define A1 (0.8f)
#define A2 (-0.2f)
#define A3 (0.03809523809f)
#define A4 (-0.00357142857f)
#include "pam_oracle_impl.h"
#undef R
#undef SFX
#undef FABS
#undef COS
#undef SIN
#undef C0
#undef C1
#undef C2
#undef C3
#undef C4
#undef A1
#undef A2
#undef A3
#undef A4

/* ---------------- FP64: exact coefficients (src/utils.py:398-402, 420-423) */
#define R double
#define SFX(n) n##_f64
#define FABS fabs
#define COS cos
#define SIN sin
#define C0 (-1435.0 / 504.0)
#define C1 (8.0 / 5.0)
#define C2 (-1.0 / 5.0)
#define C3 (8.0 / 315.0)
#define C4 (-1.0 / 560.0)
#define A1 (4.0 / 5.0)
#define A2 (-1.0 / 5.0)
#define A3 (4.0 / 105.0)
#define A4 (-1.0 / 280.0)
#include "pam_oracle_impl.h"

/* Number of OpenMP threads the oracle runs with (for the CPU-baseline record). */
#ifdef _OPENMP
#include <omp.h>
int og_threads(void) { return omp_get_max_threads(); }
void og_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }
#else
int og_threads(void) { return 1; }
void og_set_threads(int n) { (void)n; }
#endif
