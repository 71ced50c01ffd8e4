/* Logging stand-in for the reference build under emulation (no output). */
#pragma once
namespace spdlog {
template <typename... A> inline void trace(A &&...) {}
template <typename... A> inline void debug(A &&...) {}
template <typename... A> inline void info(A &&...) {}
template <typename... A> inline void warn(A &&...) {}
template <typename... A> inline void error(A &&...) {}
}  // namespace spdlog
