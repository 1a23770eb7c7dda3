// atmoscudapropagator.cu -- the reference's header name (CUDAProb3++ exports it from its install tree);
// code that includes it gets the GB300 library's C++ facade with the same class names.
#pragma once
#include "../cudaprob3_gb300.hpp"
