// Learned subgrid closure of the 3D incompressible LES: the closure term
// -P[d_j tau_ij] with tau predicted pointwise by the MLP (mlp.cuh) from the
// resolved velocity-gradient tensor and the filter width.
#pragma once
#include "dd_common.cuh"
#include "plan.cuh"

namespace dd {

// Closure parameters and its scratch region, as handed to the RHS drivers.
struct LesHook {
    const dd_closure* cl;
    void* work;
    size_t wb;
};

// Scratch bytes of the closure on plan p (gradient and stress spectra, their
// grid-point values, transform workspace).
size_t les_work_bytes(const dd_plan* p);

// nc[i] += -(i k_j tau_ij)^ on the kept modes (compact complex128 layout), for
// the state y (3 velocity components, full layout, or compact when compact).
int les_closure_add(const dd_plan* p, const LesHook& h, int prec, bool compact, const void* const* y,
                    void* const* nc, cudaStream_t st);

}  // namespace dd
