// Test-only (oracle): force-included into the reference's
// subsurface_integrator.cc by oracle/Makefile, so the time(NULL) seed of its
// subsurface photon streams (subsurface_integrator.cc:248) comes from the
// harness (rh_set_time) instead of the wall clock. The reference source
// itself is compiled unmodified.
#pragma once
#include <ctime>
extern "C" time_t rh_fake_time(time_t* t);
#define time(x) rh_fake_time(x)
