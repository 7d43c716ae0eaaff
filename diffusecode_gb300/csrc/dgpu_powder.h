// Powder "complete" mode: the rod plan of powder_complete
// (discus/prog/powder.f90:1829-2593) and the h-slabs the device evaluates.
#pragma once
#include <stdint.h>

#include <vector>

#include "../../include/discus_gpu.h"

// One (h, k) rod: its points are l = (l0 dL + shift3) + i dL, i = 0..n-1.
struct PowderRod {
    int32_t ih, ik;   // loop indices: hh = ih dH + shift1, kk = ik dK + shift2
    int32_t l0, n;    // l_start and inc(1) of the rod
};

// A box of the (h, k, l) index space evaluated in one device call.  Axis 0 is
// l (fastest), axis 1 k, axis 2 h.  tab[(ih - h0) * nk + (ik - k0)] holds
// (l_start, inc(1)) of that rod, inc(1) = 0 where there is none.
struct PowderSlab {
    int32_t h0, nh, k0, nk, l0, nl;
    int64_t tab_off;   // offset of the slab's table in PowderPlan::tab (int2 entries)
};

struct PowderPlan {
    int32_t n_pkt = 0;
    std::vector<PowderRod> rods;      // in the reference's loop order
    std::vector<PowderSlab> slabs;
    std::vector<int32_t> tab;         // (l_start, inc) pairs of all slabs
    int64_t rod_points = 0, grid_points = 0;
};

// n_pkt of powder_complete (powder.f90:1957); -1 for an invalid Q range.
int32_t dgpu_powder_npkt_host(const dgpu_powder *pw);

// The rods of powder_complete for this crystal metric (rten) and ano, then the
// slabs: consecutive h planes, at least min(#planes, min_slabs) of them and
// none larger than max_points.  Returns 0, or a DGPU_ERR_* code with msg set.
int dgpu_powder_plan(const double rten[9], const dgpu_powder *pw, int ano, int min_slabs, int64_t max_points,
                     PowderPlan &plan, char *msg, size_t msg_len);
