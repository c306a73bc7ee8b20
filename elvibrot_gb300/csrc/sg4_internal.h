// sg4_internal.h -- shared host-side definitions of the SG4 library.
#pragma once
#include <cstdarg>
#include <string>
#include <vector>

#include "evr_sg4.h"

#define EVR_MAXD 24   // modes per term handled by the kernels
#define EVR_MAXN 16   // largest 1-D grid / basis size (nq, nb) per level

namespace evr {

struct Basis1D {
  int nb = 0, nq = 0;
  std::vector<double> x, w;           // grid and wrho
  std::vector<double> RGB;            // nq x nb column-major (dnRGB%d0)
  std::vector<double> RBGw;           // nb x nq column-major (dnRBGwrho%d0)
  std::vector<double> d1GG, d2GG;     // nq x nq column-major
};

struct DescSizes {
  long long sum_nb = 0, sum_nq = 0;
  long long max_nb = 0, max_nq = 0;
};

int set_error(int code, const char* fmt, ...);
int desc_sizes(const evr_sg4_desc* d, DescSizes* z);

}  // namespace evr

struct evr_sg4_basis {
  int D = 0, L = 0, LB = 0;
  std::vector<int> nb_of_l, nq_of_l;
  std::vector<evr::Basis1D> mats;     // [D*(L+1)]
  std::vector<double> cat_x, cat_RGB, cat_RBGw, cat_d1, cat_d2;
  long long N = 0, nb_SG = 0;
  std::vector<int> tab_l;
  std::vector<double> weight;
  std::vector<int> map;
};
