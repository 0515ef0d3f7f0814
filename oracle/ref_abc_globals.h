/* Settable ABC coefficients for the pinning build of the reference's
 * force_free.c (its ffA/ffB/ffC macros are mapped onto these). */
extern double refh_ffA, refh_ffB, refh_ffC;
