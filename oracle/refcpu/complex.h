/* The reference headers spell C99 complex types ("float complex") inside C++
 * translation units (inc/cuna.h:26, inc/cuna_typedefs.h:97,108), and
 * src/cuna.cpp:46 uses C99's _Complex_I.  g++ accepts the GNU spelling, so map
 * both for the reference-on-CPU build only. */
#ifndef CUNA_REFCPU_COMPLEX_H
#define CUNA_REFCPU_COMPLEX_H
#define complex _Complex
#ifndef _Complex_I
#define _Complex_I (__extension__ 1.0iF)
#endif
#endif
