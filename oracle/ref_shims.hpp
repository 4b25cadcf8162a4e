// ref_shims.hpp — project-written shims that let the reference's own C++
// sources compile as one GCC 13 translation unit (test infrastructure only).
//
//  * every standard header that `import std;` would have provided;
//  * std::println / std::print (GCC 13's libstdc++ has no <print>);
//  * the pocketfft C API used at src/math/fft.cppm:29-41, implemented by the
//    project's own mixed-radix FFT (oracle/mrfft.h) because the reference's
//    vendor/pocketfft submodule is empty;
//  * an empty pugi::xml_node so the UPF class declaration compiles (the
//    pugixml parser itself is removed by oracle/refgen.py; oracle/ref_driver.cpp fills
//    UPF objects from an in-memory registry instead).
#pragma once

#include <algorithm>
#include <array>
#include <bit>
#include <cassert>
#include <cctype>
#include <cerrno>
#include <charconv>
#include <chrono>
#include <cmath>
#include <complex>
#include <concepts>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <filesystem>
#include <format>
#include <fstream>
#include <functional>
#include <initializer_list>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numbers>
#include <numeric>
#include <optional>
#include <random>
#include <ranges>
#include <set>
#include <span>
#include <sstream>
#include <stdexcept>
#include <string>
#include <string_view>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <variant>
#include <vector>

#include "mrfft.h"

// Output of the reference's progress messages goes to stderr so that the
// driver's stdout stays machine-readable.
namespace std {
template <class... Args>
inline void print(std::format_string<Args...> fmt, Args&&... args) {
    std::string s = std::format(fmt, std::forward<Args>(args)...);
    std::fputs(s.c_str(), stderr);
}
template <class... Args>
inline void println(std::format_string<Args...> fmt, Args&&... args) {
    std::string s = std::format(fmt, std::forward<Args>(args)...);
    s.push_back('\n');
    std::fputs(s.c_str(), stderr);
}
inline void println() { std::fputc('\n', stderr); }
template <class... Args>
inline void println(std::FILE* f, std::format_string<Args...> fmt, Args&&... args) {
    std::string s = std::format(fmt, std::forward<Args>(args)...);
    s.push_back('\n');
    std::fputs(s.c_str(), f == stdout ? stderr : f);
}
}  // namespace std

// ---- pocketfft C API over mrfft ------------------------------------------
struct cfft_plan_i {
    mrfft_plan_s* p;
};
typedef cfft_plan_i* cfft_plan;

inline cfft_plan make_cfft_plan(std::size_t length) {
    auto* h = new cfft_plan_i{mrfft_make(static_cast<int>(length))};
    return h;
}
inline void destroy_cfft_plan(cfft_plan plan) {
    if (!plan) return;
    mrfft_free(plan->p);
    delete plan;
}
inline int cfft_forward(cfft_plan plan, double c[], double fct) {
    mrfft_exec(plan->p, c, -1, fct);
    return 0;
}
inline int cfft_backward(cfft_plan plan, double c[], double fct) {
    mrfft_exec(plan->p, c, +1, fct);
    return 0;
}

// ---- pugixml placeholder ---------------------------------------------------
namespace pugi {
struct xml_node {};
}  // namespace pugi
