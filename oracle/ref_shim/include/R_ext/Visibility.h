/* Stub of R_ext/Visibility.h (oracle test infrastructure). */
#ifndef SHIM_R_VISIBILITY_H
#define SHIM_R_VISIBILITY_H
#define attribute_hidden
#endif
