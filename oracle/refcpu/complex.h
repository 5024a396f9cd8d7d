/* The reference headers spell C99 complex types ("float complex") inside C++
 * translation units (inc/cuna.h:26, inc/cuna_typedefs.h:97,108).  g++ accepts
 * the GNU spelling, so map the keyword for the reference-on-CPU build only. */
#ifndef CUNA_REFCPU_COMPLEX_H
#define CUNA_REFCPU_COMPLEX_H
#define complex _Complex
#endif
