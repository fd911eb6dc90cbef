"""Drop-in counterparts of jax_lbm.core (lattice, equilibrium, collision,
streaming, boundary, forces) running on the sm_103a kernels."""
