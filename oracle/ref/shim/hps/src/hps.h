// Stand-in for the un-vendored hps serialization header.  The reference's det code only
// declares serialize/parse templates against it (nothing is instantiated); it relies on this
// header for the fixed-width integer types, which the real one pulls in.
#pragma once
#include <cstdint>
#include <cstddef>
#include <string>
#include <cassert>
