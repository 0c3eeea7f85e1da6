"""nova-gb300: GB300-native point-based POMDP backup (PBVI / Perseus) and MDP
Bellman update behind kylewray/nova's C ABI and Python wrapper.

Modules mirror the reference's python/nova package: nova_pomdp, pomdp,
nova_pomdp_pbvi, pomdp_pbvi, nova_pomdp_perseus, pomdp_perseus,
nova_pomdp_alpha_vectors, pomdp_alpha_vectors, nova_mdp, mdp, nova_mdp_vi,
mdp_vi, nova_mdp_value_function, mdp_value_function. Import them as
`nova_gb300.<module>`; each loads nova_gb300/lib/libnova.so and fails if it
has not been built.
"""

__all__ = ["nova_mdp", "mdp",
           "nova_mdp_vi", "mdp_vi",
           "nova_mdp_value_function", "mdp_value_function",
           "nova_pomdp", "pomdp",
           "nova_pomdp_pbvi", "pomdp_pbvi",
           "nova_pomdp_perseus", "pomdp_perseus",
           "nova_pomdp_alpha_vectors", "pomdp_alpha_vectors",
           "synth"]
