// gbo_sim_tree0.cu : the simulation kernels for geometries of single-leaf prims (TREE = 0).
#define GBO_SIM_TREE 0
#include "gbo_sim_forms.inl"
