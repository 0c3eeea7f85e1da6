/*
 * nova-gb300: device copies of the MDP arrays. Aggregate calls return the
 * sum of the per-array codes (mdp_model_gpu.cu:34-78).
 */
#ifndef NOVA_MDP_MODEL_GPU_H
#define NOVA_MDP_MODEL_GPU_H

#include <nova/mdp/mdp.h>

NOVA_NS_BEGIN

/* mdp_model_gpu.h:38-45 / mdp_model_gpu.cu:34-78 */
NOVA_API int mdp_initialize_gpu(MDP *mdp);
NOVA_API int mdp_uninitialize_gpu(MDP *mdp);
/* mdp_model_gpu.h:52-59 (S) */
NOVA_API int mdp_initialize_successors_gpu(MDP *mdp);
NOVA_API int mdp_uninitialize_successors_gpu(MDP *mdp);
/* mdp_model_gpu.h:66-73 (T) */
NOVA_API int mdp_initialize_state_transitions_gpu(MDP *mdp);
NOVA_API int mdp_uninitialize_state_transitions_gpu(MDP *mdp);
/* mdp_model_gpu.h:80-87 (R) */
NOVA_API int mdp_initialize_rewards_gpu(MDP *mdp);
NOVA_API int mdp_uninitialize_rewards_gpu(MDP *mdp);
/* mdp_model_gpu.h:94-101 (goals) */
NOVA_API int mdp_initialize_goals_gpu(MDP *mdp);
NOVA_API int mdp_uninitialize_goals_gpu(MDP *mdp);

NOVA_NS_END

#endif
