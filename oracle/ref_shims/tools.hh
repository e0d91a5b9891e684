// Stand-in for Backend/includes/tools/tools.hh in the comparison build: the integer aliases and
// map_blocks_to_problem (grid size = ceil(problem / threads), checked against the device's grid
// limit) that the compute translation units use, without the JSON and filesystem helpers.
#pragma once

#include <cmath>
#include <cstddef>

#include "hardware_limits.hh"
#include "logger.hh"
#include "rect.hh"

using uchar = unsigned char;
using uint = unsigned int;
using ushort = unsigned short;
using ulong = unsigned long;

inline unsigned map_blocks_to_problem(const size_t problem_size, const unsigned nb_threads)
{
    const unsigned blocks = static_cast<unsigned>(std::ceil(static_cast<float>(problem_size) / static_cast<float>(nb_threads)));
    CHECK(blocks <= get_max_blocks(), "Too many blocks required.");
    return blocks;
}

template <typename T>
bool is_between(T val, T min, T max)
{
    return min <= val && val <= max;
}
