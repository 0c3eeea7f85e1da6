/*
 * nova-gb300: C/C++ linkage helpers shared by every public header.
 *
 * The reference declares its structs inside `namespace nova` and its entry
 * points as `extern "C"`; the exported symbol names are therefore plain C
 * names. These macros keep the same names and struct layouts while letting
 * the headers also compile as C (for cgo / JNI / ctypes users).
 */
#ifndef NOVA_ABI_H
#define NOVA_ABI_H

#ifdef __cplusplus
#define NOVA_NS_BEGIN namespace nova {
#define NOVA_NS_END }
#define NOVA_EXTERN extern "C"
#else
#define NOVA_NS_BEGIN
#define NOVA_NS_END
#define NOVA_EXTERN extern
#endif

#if defined(__GNUC__)
#define NOVA_API NOVA_EXTERN __attribute__((visibility("default")))
#else
#define NOVA_API NOVA_EXTERN
#endif

#endif
