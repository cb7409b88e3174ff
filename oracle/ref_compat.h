/*
 * ORACLE — test infrastructure only.
 * Force-included ahead of the reference's CPU sources when they are compiled
 * unmodified into oracle/_ref/. The reference was written for MSVC: it relies
 * on transitive standard includes and on the MSVC intrinsic __lzcnt
 * (src/cpu/simpleBVH.cpp:36-39). Both are supplied here; nothing else changes.
 */
#pragma once
#include <cassert>
#include <climits>
#include <cstdint>
#include <limits>
#include <memory>
#include <string>

static inline unsigned int __lzcnt(unsigned int x)
{
    return x == 0u ? 32u : (unsigned int)__builtin_clz(x);
}
