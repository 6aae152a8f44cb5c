// Empty stand-in: Waveform.h includes rtac_base signal_helpers but
// Waveform_Sine does not use it.
#pragma once
