// TEST INFRASTRUCTURE ONLY.  C entry points to the reference's own
// angular-momentum functions (new_anglib.C, compiled from the reference
// tree into oracle/_ref/libanglib.so) for the bit-identity tests of this
// library's host/su2.cpp.  2j arguments, as in the reference.
#include "new_anglib.h"

extern "C" {
double ref_clebsch(int j1, int m1, int j2, int m2, int j3, int m3) { return clebsch(j1, m1, j2, m2, j3, m3); }
double ref_six_j(int a, int b, int c, int d, int e, int f) { return six_j(a, b, c, d, e, f); }
double ref_nine_j(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
  return nine_j(a, b, c, d, e, f, g, h, i);
}
}
