// Device-build stand-in for a header the reference includes (oracle only);
// the definitions it needs come from sc_ref_device_prelude.h (force-included).
#pragma once
