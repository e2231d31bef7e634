/* ORACLE build support — test infrastructure only.
 * Hand-written stand-in for the CMake-generated Config.h of SQUANDER: no vendor BLAS is
 * selected, so the reference's BLAS==0 branches (plain CBLAS calls) are compiled. */
#ifndef SQG_REF_SHIM_CONFIG_H
#define SQG_REF_SHIM_CONFIG_H
#endif
