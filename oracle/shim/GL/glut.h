// Test infrastructure only: empty stand-in for the windowing header that the
// reference's Core.h includes; no windowing symbol is used by the physics
// translation units the oracle compiles.
#pragma once
