/* TEST INFRASTRUCTURE ONLY: the oracle.  Compiled once per precision
 * (ORC_PREC = 1 float, 2 double, 3 long double) into
 * oracle/_build/liboracle_fft.so; the product never links it.
 * The algorithms and their reference citations are in fft_oracle_impl.h. */
#include "fft_oracle_impl.h"
