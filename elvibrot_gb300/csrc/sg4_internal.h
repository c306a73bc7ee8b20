// sg4_internal.h -- shared host-side definitions of the SG4 library.
#pragma once
#include <cstdarg>
#include <string>
#include <vector>

#include "evr_sg4.h"

#define EVR_MAXD 24   // modes per term handled by the kernels
#define EVR_MAXN 16   // largest 1-D grid / basis size (nq, nb) per level
#define EVR_MAXNB0 8  // channels (electronic states) per vector

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

// Two operators on one basis applied to nrhs complex vectors in one launch,
// up to the chunk partials of both ordered accumulations (part: [2][n_chunks]
// [2 nrhs] (s, c) pairs: operator 0 first, then chunk, then re/im of each
// vector); `x` is the device input block (N x nrhs complex, ld N) of every
// apply.  `transpose` applies both transposed.
struct FieldPair;
struct FieldPairView {
  long long N = 0, n_chunks = 0;
  int nrhs = 1;
  const long long* fun_chunk = nullptr;  // [N+1] first chunk of each packed function
  const void* part = nullptr;            // double2 partials
  double* x = nullptr;
};
int field_pair_create(evr_sg4_ctx* a, evr_sg4_ctx* b, int transpose, int nrhs, FieldPair** out);
void field_pair_destroy(FieldPair* f);
int field_pair_apply(FieldPair* f, void* stream);
FieldPairView field_pair_view(const FieldPair* f);
// One context applied to fixed device buffers (nrhs real columns, ld nb0*N,
// E0 = 0, Esc = 1) with a plan and scratch of its own (the work list and
// kernel evr_sg4_apply would use): a launch enqueues kernels and a
// memset only (graph-recordable).
struct BoundApply;
int bound_apply_create(evr_sg4_ctx* c, int nrhs, int transpose, const double* psi, double* hpsi, BoundApply** out);
int bound_apply_launch(BoundApply* b, void* stream);
void bound_apply_destroy(BoundApply* b);
// A multi-context plan's parameter blocks bound to fixed vectors (slot 0 or
// 1, ld = nb0*N): a bound launch enqueues kernels and memsets only.
int multi_bind(evr_sg4_multi* m, int slot, const double* const* psi, double* const* hpsi);
int multi_launch_bound(evr_sg4_multi* m, int slot, const double* const* psi, double* const* hpsi, const double* E0,
                       const double* Esc, void* stream);
// Contexts, right-hand sides per context, complex shift and transpose flag
// of a multi-context plan.
void multi_shape(const evr_sg4_multi* m, std::vector<evr_sg4_ctx*>* ctxs, std::vector<int>* nrhs, int* cshift,
                 int* transpose);

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
