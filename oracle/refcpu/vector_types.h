/* Host-only stand-in for <vector_types.h> (reference-on-CPU build only). */
#ifndef CUNA_REFCPU_VECTOR_TYPES_H
#define CUNA_REFCPU_VECTOR_TYPES_H
struct float2 { float x, y; };
struct double2 { double x, y; };
typedef struct float2 float2;
typedef struct double2 double2;
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
#endif
