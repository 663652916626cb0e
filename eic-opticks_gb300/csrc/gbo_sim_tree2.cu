// gbo_sim_tree2.cu : the simulation kernels for geometries with CSG list nodes (TREE = 2).
#define GBO_SIM_TREE 2
#include "gbo_sim_forms.inl"
