// The tile-pass kernels for lsg::DF elements (see kernels.cuh).
#include "kernels_impl.cuh"

template struct lsg::PassKernels<lsg::DF>;
