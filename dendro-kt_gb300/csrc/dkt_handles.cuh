// The opaque handles of the C ABI (include/dkt_gb300.h).
#pragma once
#include "dkt_internal.cuh"

struct dkt_da_s {
  dkt::DA da;
};
struct dkt_plan_s {
  dkt::Plan pl;
};
