// The opaque handle types of include/gpetsc.h (one definition, shared by the
// translation units that implement the C ABI).
#pragma once

#include "gp_ksp.h"

struct gp_mat_s {
  gp::Csr* A;
};
struct gp_pc_s {
  gp::Pc* pc;
};
struct gp_ksp_s {
  gp::Ksp* k;
};
