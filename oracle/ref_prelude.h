/*
 * Force-included when compiling the reference FDTD into oracle/_ref/libref_fdtd.so
 * (TEST INFRASTRUCTURE ONLY).  Turns the reference's exit() calls into a
 * counter so that a check that would end the process (e.g. the monitor-plane
 * guard of main_calc, FDTDsplitfieldMetal.c:320) is reported to the caller
 * instead of killing the Python test process.  The stock binary _ref/FDTD_ref
 * is built without it.
 */
#include <stdlib.h>
void ref_soft_exit(int code);
#define exit(code) ref_soft_exit(code)
