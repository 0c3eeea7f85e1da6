/*
 * nova-gb300: device copies of the POMDP arrays.
 *
 * Each per-array pair allocates and uploads (or frees) one d_* field; the
 * aggregate calls return the SUM of the per-array codes, as the reference
 * does (pomdp_model_gpu.cu:34-75).
 */
#ifndef NOVA_POMDP_MODEL_GPU_H
#define NOVA_POMDP_MODEL_GPU_H

#include <nova/pomdp/pomdp.h>

NOVA_NS_BEGIN

/* pomdp_model_gpu.h:38 / pomdp_model_gpu.cu:34-53 */
NOVA_API int pomdp_initialize_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:45 / pomdp_model_gpu.cu:56-75 */
NOVA_API int pomdp_uninitialize_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:52-59 / pomdp_model_gpu.cu:78-122 (S) */
NOVA_API int pomdp_initialize_successors_gpu(POMDP *pomdp);
NOVA_API int pomdp_uninitialize_successors_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:66-73 / pomdp_model_gpu.cu:125-168 (T) */
NOVA_API int pomdp_initialize_state_transitions_gpu(POMDP *pomdp);
NOVA_API int pomdp_uninitialize_state_transitions_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:80-87 / pomdp_model_gpu.cu:171-214 (O) */
NOVA_API int pomdp_initialize_observation_transitions_gpu(POMDP *pomdp);
NOVA_API int pomdp_uninitialize_observation_transitions_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:94-101 / pomdp_model_gpu.cu:217-260 (R) */
NOVA_API int pomdp_initialize_rewards_gpu(POMDP *pomdp);
NOVA_API int pomdp_uninitialize_rewards_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:108-115 / pomdp_model_gpu.cu:263-307 (Z) */
NOVA_API int pomdp_initialize_nonzero_beliefs_gpu(POMDP *pomdp);
NOVA_API int pomdp_uninitialize_nonzero_beliefs_gpu(POMDP *pomdp);
/* pomdp_model_gpu.h:122-129 / pomdp_model_gpu.cu:310-353 (B) */
NOVA_API int pomdp_initialize_belief_points_gpu(POMDP *pomdp);
NOVA_API int pomdp_uninitialize_belief_points_gpu(POMDP *pomdp);

NOVA_NS_END

#endif
