// TEST INFRASTRUCTURE: declaration only (lattice/tensor.h names the type).
#pragma once
namespace util {
template <class R, int W> struct simd;
}
