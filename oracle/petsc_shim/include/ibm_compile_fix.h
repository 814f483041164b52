/*
 * TEST INFRASTRUCTURE ONLY.  Forced-included (gcc -include) when the reference's
 * ibm.c is compiled for the oracle's pinning library.  ibm.c declares
 * point_cell_thin with 19 parameters (ibm.c:12) but defines it with 13
 * (ibm.c:1413), which no C compiler accepts.  This macro gives the two forms
 * distinct names by their argument count (point_cell_thin_19 / _13), so the
 * file compiles unmodified.  point_cell_thin serves thin bodies only; the
 * classification path (ibm_search_advanced, point_cell_advanced) never calls it.
 */
#ifndef CVB_IBM_COMPILE_FIX_H
#define CVB_IBM_COMPILE_FIX_H
#define CVB_NARGS(...) CVB_NARGS_(__VA_ARGS__, 24, 23, 22, 21, 20, 19, 18, 17, 16, 15, 14, 13, 12, 11, 10, 9, 8, \
                                  7, 6, 5, 4, 3, 2, 1)
#define CVB_NARGS_(a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15, a16, a17, a18, a19, a20, \
                   a21, a22, a23, a24, N, ...) N
#define CVB_CAT(a, b) CVB_CAT_(a, b)
#define CVB_CAT_(a, b) a##b
#define point_cell_thin(...) CVB_CAT(point_cell_thin_, CVB_NARGS(__VA_ARGS__))(__VA_ARGS__)
#endif
