// The (nx, ny) pairs with compiled kernels, as X-macro lists.  Each
// instantiation file (inst_<dtype>_<nx>_<ny>.cu) builds one pair.
#pragma once
#define SS_FOR_SMALL_DIMS(X) \
  X(1, 1) X(1, 2) X(1, 3) \
  X(2, 1) X(2, 2) X(2, 3) \
  X(3, 1) X(3, 2) X(3, 3) \
  X(4, 1) X(4, 2) X(4, 3) \
  X(5, 1) X(5, 2) X(5, 3)
// Six- to eight-state models (thread-per-chunk kernels as for nx <= 5; FP64 at these
// sizes runs the unstaged kernels, whose records do not fit the staging tiles).
#define SS_FOR_WIDE_DIMS(X) \
  X(6, 1) X(6, 2) X(6, 3) \
  X(7, 1) X(7, 2) \
  X(8, 1) X(8, 2)
#define SS_FOR_DIMS(X) SS_FOR_SMALL_DIMS(X) SS_FOR_WIDE_DIMS(X)
// (nx, ny) pairs with forward-mode gradient kernels (ss_filter_grad).
#define SS_FOR_GRAD_DIMS(X) X(2, 2) X(5, 2)
// (nx, ny) pairs with reverse-mode gradient kernels (ss_filter_adjoint).
#define SS_FOR_ADJ_DIMS(X) SS_FOR_SMALL_DIMS(X)
// (nx, ny) pairs of the large-state (dense, warp-per-item) path for linear models.
#define SS_FOR_DENSE_DIMS(X) X(8, 4) X(32, 16)
#define SS_MAX_NX 5
#define SS_MAX_NY 3
