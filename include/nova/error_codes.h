/*
 * nova-gb300: status codes returned by every entry point.
 *
 * The numeric values are part of the ABI and equal those of the reference
 * (include/nova/error_codes.h:32-48). NOVA_CONVERGED is a non-error status
 * returned by the Perseus update when the set of beliefs still to improve is
 * empty.
 */
#ifndef NOVA_ERROR_CODES_H
#define NOVA_ERROR_CODES_H

#define NOVA_SUCCESS                                0

#define NOVA_ERROR_INVALID_DATA                     1
#define NOVA_ERROR_INVALID_CUDA_PARAM               2
#define NOVA_ERROR_DEVICE_MALLOC                    3
#define NOVA_ERROR_MEMCPY_TO_DEVICE                 4
#define NOVA_ERROR_MEMCPY_TO_HOST                   5
#define NOVA_ERROR_DEVICE_FREE                      6
#define NOVA_ERROR_KERNEL_EXECUTION                 7
#define NOVA_ERROR_DEVICE_SYNCHRONIZE               8

#define NOVA_CONVERGED                              9
#define NOVA_WARNING_INVALID_BELIEF                 10
#define NOVA_ERROR_OUT_OF_MEMORY                    11
#define NOVA_ERROR_POLICY_CREATION                  12

#endif
