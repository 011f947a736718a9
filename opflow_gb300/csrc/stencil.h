// Tiled axis-stencil kernels (u_out = f(u at i, i +- e_d)) shared by the expression lowering.
#pragma once
#include "internal.h"

#include <type_traits>

namespace opg {

struct AxisParams {
    int ndim;
    // EXACT: u + s * (d2<order[0]> + d2<order[1]> [+ d2<order[2]>]) with spacing h per dim
    double h[3], inv_h[3];
    int pow2[3];
    int order[3];
    double s;
    // FAST: u + sum_d w_d * ((u(i-e_d) - u) + (u(i+e_d) - u)) in fixed point
    int iso;                     // one weight for every dim (w[0])
    unsigned long long wm[3];    // weight mantissas
    int wshift[3], wneg[3];
    unsigned long long bound_bits;
};

int axis_launch(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P, bool fast,
                unsigned long long* maxslots, int step);
// One step of a run of fixed-point steps that keeps the update box in fixed point between steps (2D or
// 3D; in 3D the steady-state steps stage their planes by TMA where the buffer's strides allow):
// `first` reads float64, `last` writes float64; maxslots[0] holds the initial max|u| bit pattern.
bool axis_resident_ok(const AxisParams& P);  // weights the resident kernel's product takes
int axis_launch_resident(opflow_ctx ctx, const FieldView& in, const FieldView& out, const Box& box, const AxisParams& P,
                         const unsigned long long* maxslots, bool first, bool last);
// Reads and clears the flag a TMA-staged step sets when one of its bounded waits gave up.
int stencil_take_error(cudaStream_t s, int* err);

}  // namespace opg
