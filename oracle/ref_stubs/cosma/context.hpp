// Stand-in for the reference's context header on a CPU build: the context
// types appear only as arguments that the CPU path of local_multiply passes on.
#pragma once
#include <iostream>  // the real header chain brings it; local_multiply.cpp prints with std::cout
#include <memory>
namespace cosma {
template <typename Scalar>
class cosma_context {};
template <typename Scalar>
using context = std::unique_ptr<cosma_context<Scalar>>;
template <typename Scalar>
cosma_context<Scalar>* get_context_instance();
}  // namespace cosma
