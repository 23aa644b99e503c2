// The tile-pass kernels for double elements (see kernels.cuh).
#include "kernels_impl.cuh"

template struct lsg::PassKernels<double>;
