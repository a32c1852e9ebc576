// Lattice constants for the device and host code of the GB300 LBM library.
//
// Direction order, weights and opposite tables are the reference's
// (src/lbm/constants.h:247-365): the reference's neighbour table is indexed by
// these direction ids, so they cannot be renumbered.  The rest direction is
// the LAST one.  D3Q7 (absent from the reference) follows the same
// convention: six face neighbours in (-x,+x,-y,+y,-z,+z) order, rest last.
#pragma once

#include "../../include/lbm_gpu.h"

#define LBM_HD __host__ __device__ __forceinline__

namespace lbm {

constexpr double CSSQ = 1.0 / 3.0;  // lbm_cssq, src/lbm/constants.h:27

template <int LAT>
struct Lattice;

template <>
struct Lattice<LBM_D1Q3> {
  static constexpr int D = 1, Q = 3, NNGHBR = 2;
  static LBM_HD constexpr int c(int q, int d) {
    constexpr int t[3] = {-1, 1, 0};
    return d == 0 ? t[q] : 0;
  }
  static LBM_HD constexpr int opp(int q) {
    constexpr int t[3] = {1, 0, 2};
    return t[q];
  }
  static LBM_HD constexpr double w(int q) { return q == 2 ? 2.0 / 3.0 : 1.0 / 6.0; }
  static constexpr double poisson_alpha = 1.0 / 3.0;
  static LBM_HD constexpr double pw(int q) { return q == 2 ? 0.0 : 0.5; }
};

template <>
struct Lattice<LBM_D2Q5> {
  static constexpr int D = 2, Q = 5, NNGHBR = 8;
  static LBM_HD constexpr int c(int q, int d) {
    constexpr int t[5][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {0, 0}};
    return d < 2 ? t[q][d] : 0;
  }
  static LBM_HD constexpr int opp(int q) {
    constexpr int t[5] = {1, 0, 3, 2, 4};
    return t[q];
  }
  static LBM_HD constexpr double w(int q) { return q == 4 ? 1.0 / 3.0 : 1.0 / 6.0; }
  static constexpr double poisson_alpha = 1.0 / 2.0;
  static LBM_HD constexpr double pw(int q) { return q == 4 ? 0.0 : 0.25; }
};

template <>
struct Lattice<LBM_D2Q9> {
  static constexpr int D = 2, Q = 9, NNGHBR = 8;
  static LBM_HD constexpr int c(int q, int d) {
    constexpr int t[9][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {1, 1}, {1, -1}, {-1, -1}, {-1, 1}, {0, 0}};
    return d < 2 ? t[q][d] : 0;
  }
  static LBM_HD constexpr int opp(int q) {
    constexpr int t[9] = {1, 0, 3, 2, 6, 7, 4, 5, 8};
    return t[q];
  }
  static LBM_HD constexpr double w(int q) { return q == 8 ? 4.0 / 9.0 : (q < 4 ? 1.0 / 9.0 : 1.0 / 36.0); }
  static constexpr double poisson_alpha = 1.0 / 3.0;
  static LBM_HD constexpr double pw(int q) { return q == 8 ? 0.0 : 1.0 / 8.0; }
};

template <>
struct Lattice<LBM_D3Q7> {
  static constexpr int D = 3, Q = 7, NNGHBR = 6;
  static LBM_HD constexpr int c(int q, int d) {
    constexpr int t[7][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}, {0, 0, 0}};
    return d < 3 ? t[q][d] : 0;
  }
  static LBM_HD constexpr int opp(int q) {
    constexpr int t[7] = {1, 0, 3, 2, 5, 4, 6};
    return t[q];
  }
  // D3Q7 Poisson lattice in the form of Chai & Shi (2008): w_0 = 1/4 at rest,
  // the six links share the rest equally; alpha = c_s^2-like constant 1/4
  static LBM_HD constexpr double w(int q) { return q == 6 ? 1.0 / 4.0 : 1.0 / 8.0; }
  static constexpr double poisson_alpha = 1.0 / 4.0;
  static LBM_HD constexpr double pw(int q) { return q == 6 ? 0.0 : 1.0 / 6.0; }
};

template <>
struct Lattice<LBM_D3Q19> {
  static constexpr int D = 3, Q = 19, NNGHBR = 18;
  static LBM_HD constexpr int c(int q, int d) {
    constexpr int t[19][3] = {{-1, 0, 0},  {1, 0, 0},  {0, -1, 0},  {0, 1, 0},  {0, 0, -1}, {0, 0, 1},  {-1, -1, 0},
                              {-1, 1, 0},  {1, -1, 0}, {1, 1, 0},   {-1, 0, -1}, {-1, 0, 1}, {1, 0, -1},  {1, 0, 1},
                              {0, -1, -1}, {0, -1, 1}, {0, 1, -1},  {0, 1, 1},   {0, 0, 0}};
    return d < 3 ? t[q][d] : 0;
  }
  static LBM_HD constexpr int opp(int q) {
    constexpr int t[19] = {1, 0, 3, 2, 5, 4, 9, 8, 7, 6, 13, 12, 11, 10, 17, 16, 15, 14, 18};
    return t[q];
  }
  static LBM_HD constexpr double w(int q) { return q == 18 ? 1.0 / 3.0 : (q < 6 ? 1.0 / 18.0 : 1.0 / 36.0); }
  static constexpr double poisson_alpha = 0.0;
  static LBM_HD constexpr double pw(int q) { return q == 18 ? 0.0 : 1.0 / 18.0; }
};

}  // namespace lbm
