// Device-build path to the jsoncpp stand-in (oracle only): the same one the
// host build uses (shim/json/json.h).
#pragma once
#include "../../shim/json/json.h"
