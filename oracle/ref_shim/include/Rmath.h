/* Stub of Rmath.h (oracle test infrastructure): the files compiled here
 * call nothing from it. */
#ifndef SHIM_RMATH_H
#define SHIM_RMATH_H
#endif
