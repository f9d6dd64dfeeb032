// TEST INFRASTRUCTURE ONLY: the kernel headers name torch::Tensor only in
// host wrappers that the emulation does not compile.
#pragma once
namespace torch {
struct Tensor {};
}
namespace at {
enum class ScalarType { Bool, Int, Float, Double };
}
