// The tile-pass kernels for lsg::Cx<double> elements (see kernels.cuh).
#include "kernels_impl.cuh"

template struct lsg::PassKernels<lsg::Cx<double>>;
