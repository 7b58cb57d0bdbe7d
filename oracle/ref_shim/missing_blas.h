/* Stand-in for the external BLAS routines that parts of the reference's
 * supernodal solves call; the build routes them here (see oracle/build.py)
 * and the stub aborts, since no BLAS is built. */
#pragma once
extern "C" void ref_blas_missing(...);
