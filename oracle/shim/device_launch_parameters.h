// Host-build stand-in for a CUDA header the reference includes; the
// definitions it needs come from sc_ref_prelude.h (force-included).
#pragma once
