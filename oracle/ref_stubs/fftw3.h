/* Build-only stand-in for <fftw3.h>: src/utils/lib_image.h includes it but the
 * compiled path uses none of its declarations.  TEST INFRASTRUCTURE ONLY. */
#ifndef BM4DOF_REF_STUB_FFTW3_H
#define BM4DOF_REF_STUB_FFTW3_H
#endif
