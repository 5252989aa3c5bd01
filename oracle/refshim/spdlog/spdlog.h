// Stand-in for spdlog (TEST INFRASTRUCTURE for oracle/_ref): logging calls are accepted and dropped.
#pragma once
namespace spdlog {
template <class... A> inline void critical(A &&...) {}
template <class... A> inline void error(A &&...) {}
template <class... A> inline void warn(A &&...) {}
template <class... A> inline void info(A &&...) {}
template <class... A> inline void debug(A &&...) {}
} // namespace spdlog
