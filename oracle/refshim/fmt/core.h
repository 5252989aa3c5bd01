// Stand-in for fmt (TEST INFRASTRUCTURE for oracle/_ref): the reference only prints iteration counts.
#pragma once
#include <string>
namespace fmt {
template <class... A> inline std::string format(A &&...) { return std::string(); }
template <class... A> inline void print(A &&...) {}
} // namespace fmt
