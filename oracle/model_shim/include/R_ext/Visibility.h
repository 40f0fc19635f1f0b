/* Stub of R_ext/Visibility.h (oracle test infrastructure). */
#ifndef SHIM_MODEL_VISIBILITY_H
#define SHIM_MODEL_VISIBILITY_H
#define attribute_hidden
#endif
