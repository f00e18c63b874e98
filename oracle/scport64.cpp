// scport64.cpp -- TEST INFRASTRUCTURE ONLY: the FP64 host oracle.
//
// The CPU restatement of the step (oracle/scport.cpp) built with every
// floating-point quantity a double (SC_PORT_FP64, oracle/scmath64.h): the
// same algorithm -- the reference's kernels in its launch order, the same
// noise draws keyed by (seed, particle id, step), the same rules and
// constants -- evaluated in double precision.  It is the reference of the
// ensemble criterion: the single-precision step's mean squared displacement
// and pair-distance histogram after many steps must fall within 1 % of this
// build's on the same initial states.  Its trajectories are not the
// single-precision ones bit for bit (the rounding differs from the first
// step on, and neighbour dynamics amplify it), which is what makes the
// comparison a test of the single-precision arithmetic.
#define SC_PORT_FP64 1
#include "scport.cpp"
