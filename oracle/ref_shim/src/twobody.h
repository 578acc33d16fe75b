/* Stand-in for twobody's src/twobody.h, which the reference's Cython module
 * includes (thejoker/src/fast_likelihood.pyx:27-30).  The function body is the
 * oracle's own Kepler solver (oracle/kepler.c). */
#include "../../kepler.h"
