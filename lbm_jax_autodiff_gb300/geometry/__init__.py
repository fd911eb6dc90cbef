"""Drop-in counterparts of jax_lbm.geometry (sphere / box / mask q builders,
sigmoid porosity, soft bounce-back) on the sm_103a kernels."""
