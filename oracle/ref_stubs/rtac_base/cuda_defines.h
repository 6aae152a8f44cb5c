// Minimal host-only stand-in for the non-vendored rtac_base header of the same
// name. It exists so that the reference's header-only arithmetic (Binner::Key,
// Waveform_Sine) can be compiled unmodified with g++ to produce golden vectors.
#pragma once
#define RTAC_HOSTDEVICE
