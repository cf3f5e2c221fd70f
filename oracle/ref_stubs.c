/*
 * ref_stubs.c -- test infrastructure (oracle), linked only into the reference
 * library oracle/_ref/libyael_ref.so.
 *
 * yael/matrix.c is compiled into that library for fmat_mul_tr, which yael/gmm.c
 * calls.  matrix.c also refers to LAPACK (sgels_, sgeqrf_, slarfb_, slarft_)
 * and to yael/eigs.c / ARPACK entry points that no function under test reaches
 * and that no library here provides.  These definitions only let the loader
 * resolve the library: each one prints its name and aborts if it is ever called.
 */
#include <stdio.h>
#include <stdlib.h>

#define REF_STUB(name)                                                           \
  void name(void)                                                                \
  {                                                                              \
    fprintf(stderr, "oracle/_ref: %s is not available in this build\n", #name);  \
    abort();                                                                     \
  }

REF_STUB(sgels_)
REF_STUB(sgeqrf_)
REF_STUB(slarfb_)
REF_STUB(slarft_)
REF_STUB(eigs_sym)
REF_STUB(eigs_sym_part)
REF_STUB(eigs_reorder)
REF_STUB(arpack_eigs_begin)
REF_STUB(arpack_eigs_step)
REF_STUB(arpack_eigs_end)
