// Minimal stand-in for Mt-KaHyPar's scalable_vector (a TBB-allocated vector
// there, a std::vector here).
#pragma once

#include <vector>

namespace mt_kahypar {
namespace parallel {
template <typename T>
using scalable_vector = std::vector<T>;
}  // namespace parallel
}  // namespace mt_kahypar
