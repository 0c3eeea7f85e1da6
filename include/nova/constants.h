/*
 * nova-gb300: numeric sentinels.
 *
 * nova replaces FLT_MAX / FLT_MIN by +1e10 / -1e10 and uses them as the start
 * value of every argmax (include/nova/constants.h:33-35). Code that includes
 * this header sees the same macros; the library itself uses the NOVA_ names.
 */
#ifndef NOVA_CONSTANTS_H
#define NOVA_CONSTANTS_H

#define NOVA_FLT_MAX      1e+10f
#define NOVA_FLT_MIN      (-1e+10f)
#define NOVA_FLT_ERR_TOL  1e-9

#ifndef NOVA_KEEP_SYSTEM_FLT
#undef FLT_MAX
#undef FLT_MIN
#define FLT_MAX 1e+10
#define FLT_MIN -1e+10
#define FLT_ERR_TOL 1e-9
#endif

#endif
