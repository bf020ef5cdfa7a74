// Minimal fmt subset on std::format — TEST INFRASTRUCTURE for compiling the reference's sources
// in the oracle build (they use fmt::format, fmt::print, fmt::runtime).
#pragma once
#include <cstdio>
#include <format>
#include <string>
#include <string_view>

namespace fmt {
struct runtime_string { std::string_view s; };
inline runtime_string runtime(std::string_view s) { return { s }; }
template <typename... A> std::string format(std::format_string<A...> f, A &&...a) { return std::format(f, std::forward<A>(a)...); }
inline std::string format(runtime_string r) { return std::string(r.s); }
template <typename... A> void print(std::format_string<A...> f, A &&...a) { std::fputs(std::format(f, std::forward<A>(a)...).c_str(), stdout); }
inline void print(runtime_string r) { std::fwrite(r.s.data(), 1, r.s.size(), stdout); }
}  // namespace fmt
