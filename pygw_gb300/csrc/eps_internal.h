// Steps of the ε block shared by the FP64 and the mixed-precision inverse
// (internal interface, not part of the C-ABI).  Layout: eps[I + N·J + N²·ω].
#pragma once
#include <cuda_runtime.h>

namespace pge {

// eps ← (eps + epsᴴ)/2 + I for every frequency (pygw.py:3229-3232).
void launch_sym_add_identity(double2* eps, int N, int nom, cudaStream_t s);

// On ε⁻¹ in eps: the q = 0 head/wings update when epsw1 is non-null
// (pygw.py:3246-3263; bw1/w2b are [nom][N] scratch), then eps −= I.
void launch_finish(double2* eps, int N, int nom, double2* epsw1, double2* epsw2, double2* head, double2* bw1,
                   double2* w2b, cudaStream_t s);

}  // namespace pge
