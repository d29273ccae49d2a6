// wdem_variant.h -- the two arithmetic variants of the step kernels.
//
// k_contact.cu and k_leapfrog.cu are compiled twice.  As written (--fmad=false) every FP64 operation is
// the IEEE operation of the reference's expression, in its order: results equal the CPU restatement bit
// for bit.  With WDEM_FMA defined (--fmad=true) multiply-adds are contracted into FMAs and a division of
// a vector by a scalar takes one reciprocal; those kernels and launchers live in namespace
// wdem::contracted, and the host selects them with wdem_params.arith = WDEM_ARITH_FMA, or WDEM_ARITH_DW
// (the contracted kernels with the double-word contact law of k_contact.cu, StepParams.dw).
#pragma once
#ifdef WDEM_FMA
#define WDEM_VARIANT_BEGIN namespace contracted {
#define WDEM_VARIANT_END }
#else
#define WDEM_VARIANT_BEGIN
#define WDEM_VARIANT_END
#endif
