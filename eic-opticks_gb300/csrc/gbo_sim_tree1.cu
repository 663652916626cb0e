// gbo_sim_tree1.cu : the simulation kernels for geometries with CSG boolean trees (TREE = 1).
#define GBO_SIM_TREE 1
#include "gbo_sim_forms.inl"
