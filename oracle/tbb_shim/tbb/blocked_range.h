// Stand-in for TBB's blocked_range over an integer interval (used by
// src/omp_lattice.cpp:115,364,402).  Oracle build only.
#pragma once
#include <cstddef>
namespace tbb {
template <typename T> class blocked_range {
public:
    blocked_range(T b, T e) : m_b(b), m_e(e) {}
    T begin() const { return m_b; }
    T end() const { return m_e; }
private:
    T m_b, m_e;
};
}
