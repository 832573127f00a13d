// wf_mlp.cu — placeholder translation unit for the MLP training kernels.
#include "wf_mlp.cuh"
