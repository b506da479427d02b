/*
 * gl_oracle.h -- CPU restatement of the mepgl hot path (TEST INFRASTRUCTURE).
 *
 * This is the oracle against which the CUDA library is checked.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product path never does.  Each function cites the reference code it
 * restates (paths relative to the maiani/mepgl tree).  Parity of this
 * restatement with the reference's own kernels is established by
 * tests/test_oracle_vs_ref.py (host-compiled reference kernels, built by
 * oracle/ref_build.py) and by the golden vectors in tests/golden/.
 *
 * Layout: site (i, j) of image n at i + nx*j + nx*ny*n (x fastest); vector
 * and complex fields are interleaved (x, y) / (Re, Im) pairs, i.e. the
 * reference's real2 device layout.  Per-image scalars are double.
 *
 * The implementation (gl_oracle_impl.h) is instantiated for double (suffix
 * _d) and float (suffix _f); the exported symbols are listed in gl_oracle.c.
 */
#ifndef MEPGL_GL_ORACLE_H
#define MEPGL_GL_ORACLE_H

#include <stdint.h>

/* Options of the line search and spline (mirrors include/mepgl.h). */
enum { GLO_LS_COMPAT = 0, GLO_LS_EXACT = 1 };
enum { GLO_SPLINE_COMPAT = 0, GLO_SPLINE_FMM = 1 };
enum { GLO_METRIC_FIELDS = 0, GLO_METRIC_JB = 1 };

#endif
