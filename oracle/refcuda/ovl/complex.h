/* Overlay of <complex.h> for compiling the reference library's sources as
 * C++ (oracle/build_ref_cuda.py): its headers spell C99 complex types
 * ("float complex", inc/cuna.h:26, inc/cuna_typedefs.h:40,51), which C++'s
 * <complex.h> does not define; the GNU spelling "_Complex" is what the
 * reference meant.  Test infrastructure only. */
#include_next <complex.h>
#undef complex
#define complex _Complex
