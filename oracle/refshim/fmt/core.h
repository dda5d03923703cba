// Stand-in for the fmt library: every print / sprintf compiles to nothing
// (test infrastructure).
#pragma once
#include <cstdio>
#include <string>
namespace fmt {
enum class color { steel_blue, floral_white, medium_violet_red, forest_green };
enum class emphasis { bold };
struct text_style {};
inline text_style fg(color) { return {}; }
inline text_style operator|(text_style s, emphasis) { return s; }
template <typename... A>
void print(A &&...) {}
template <typename... A>
std::string sprintf(A &&...) { return std::string(); }
template <typename... A>
std::string format(A &&...) { return std::string(); }
}  // namespace fmt
