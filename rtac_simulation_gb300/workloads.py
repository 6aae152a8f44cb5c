"""Seeded synthetic sensors and echo-sample buffers.

The reference measures nothing itself and its demos need private meshes and
rosbags, so every workload here is synthetic: seeded numpy generators with the
shapes, sizes and value distributions of the benchmark configurations
(1D EA400-like, 2D Oculus-like, the dense 512-bearing precision ping, the
batched mixed-sensor set and the contention stress ping).

Tables follow the reference where it defines them:
  * ``waveform_sine``  Waveform_Sine (include/rtac_simulation/Waveform.h:96-138)
  * ``arcsin_bearings`` the law of examples/oculus_M1200d_1_bearings.csv
    (theta_k = asin(sin(aperture / 2) * (2k / (n - 1) - 1)))
  * ``adaptive_duration`` SensorInstance::set_ranges (src/SensorInstance.cu:26-27)
Pulses "sampled at bin spacing" and sinc-squared beams are the benchmark's own
table definitions; BeamDirectivity_Sinc's table comes from the non-vendored
rtac_base SincFunction, so ``beam_sinc`` is a stand-in with the same role.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32
DEG = math.pi / 180.0


def linspace_resolution(rmin: float, rmax: float, n: int) -> np.float32:
    """rtac Linspace resolution (max - min) / (n - 1), in float."""
    return F32(F32(F32(rmax) - F32(rmin)) / F32(n - 1))


def linspace(rmin: float, rmax: float, n: int) -> np.ndarray:
    """Output range of each bin: min + r * resolution, in float."""
    if n <= 1:
        return np.array([rmin], dtype=F32)
    res = linspace_resolution(rmin, rmax, n)
    return (F32(rmin) + (np.arange(n, dtype=F32) * res).astype(F32)).astype(F32)


def waveform_sine(frequency: float, duration: float, oversampling: int = 8) -> np.ndarray:
    """Waveform_Sine table: size = (unsigned)(2 f os * duration) in float,
    w[i] = (cos phase, sin phase) with phase = (float)(i * (2 pi f / fs))."""
    f = F32(frequency)
    fs = F32(F32(2.0) * f * F32(oversampling))
    size = int(np.floor(F32(fs * F32(duration))))
    step = 2.0 * math.pi * float(f) / float(fs)
    phase = (np.arange(size, dtype=np.float64) * step).astype(F32)
    return (np.cos(phase.astype(np.float64)) + 1j * np.sin(phase.astype(np.float64))).astype(np.complex64)


def adaptive_duration(rmin: float, rmax: float, n: int, c: float) -> np.float32:
    """Adaptive pulse duration: Linspace resolution / c (src/SensorInstance.cu:26-27)."""
    return F32(linspace_resolution(rmin, rmax, n) / F32(c))


def arcsin_bearings(n: int, aperture_deg: float) -> np.ndarray:
    k = np.arange(n, dtype=np.float64)
    return np.arcsin(math.sin(0.5 * aperture_deg * DEG) * (2.0 * k / (n - 1) - 1.0)).astype(F32)


def texel_centers(n: int, span: float) -> np.ndarray:
    """Abscissa of each texel centre of an n-tap table spanning [-span/2, span/2]."""
    return ((np.arange(n, dtype=np.float64) + 0.5) / n - 0.5) * span


def pulse_at_bin_spacing(taps: int, res: float, frequency: float, c: float) -> np.ndarray:
    """Complex Gaussian-windowed tone burst with one tap per range bin.

    Tap k sits at range offset d_k = (k - (taps - 1) / 2) * res; the tone is the
    two-way carrier exp(i 4 pi f d / c) and the window sigma is taps * res / 6.
    """
    d = (np.arange(taps, dtype=np.float64) - (taps - 1) / 2.0) * res
    sigma = taps * res / 6.0
    w = np.exp(-0.5 * (d / sigma) ** 2) * np.exp(1j * 4.0 * math.pi * frequency * d / c)
    return w.astype(np.complex64)


def beam_sinc2(taps: int, span: float, resolution: float, floor: float = 0.0) -> np.ndarray:
    """Sinc-squared beam table (first null at `resolution`), optionally floored."""
    x = texel_centers(taps, span)
    b = np.sinc(x / resolution) ** 2
    if floor > 0.0:
        b = np.maximum(b, floor)
    return b.astype(F32)


def beam_sinc(span: float, resolution: float, oversampling: int = 8) -> np.ndarray:
    """Stand-in for BeamDirectivity_Sinc (include/rtac_simulation/BeamDirectivity.h:94-99):
    a sinc with its first null at `resolution`, `oversampling` taps per
    resolution cell, over `span`."""
    taps = 2 * int(round(0.5 * oversampling * span / resolution)) + 1
    return np.sinc(texel_centers(taps, span) / resolution).astype(F32)


@dataclass
class Workload:
    name: str
    dims: int
    sensor: dict
    samples: np.ndarray               # (N, 3) SimSample1D or (N, 4) SimSample2D, float32
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.samples.shape[0])

    @property
    def out_shape(self) -> tuple:
        if self.dims == 1:
            return (self.sensor["range_count"],)
        return (self.sensor["range_count"], len(self.sensor["bearings"]))


def _rayleigh_phasor(rng: np.random.Generator, n: int, sigma: float = 1.0):
    a = rng.rayleigh(sigma, n)
    ph = rng.uniform(0.0, 2.0 * math.pi, n)
    return a * np.cos(ph), a * np.sin(ph)


def _pack(re, im, travel, bearing=None) -> np.ndarray:
    cols = [re, im, travel] + ([bearing] if bearing is not None else [])
    out = np.empty((len(travel), len(cols)), dtype=F32)
    for i, c in enumerate(cols):
        out[:, i] = c
    return out


def sensor_1d(rmin, rmax, n_ranges, c, pulse, extent) -> dict:
    duration = F32(F32(extent) / F32(c))
    return dict(range_min=float(rmin), range_max=float(rmax), range_count=int(n_ranges),
                sound_celerity=float(c), pulse_duration=float(duration),
                margin=float(F32(F32(c) * duration)), pulse=pulse)


def sensor_2d(rmin, rmax, n_ranges, c, pulse, extent, beam, span, bearings) -> dict:
    s = sensor_1d(rmin, rmax, n_ranges, c, pulse, extent)
    s.update(beam=beam, beam_span=float(span), bearings=bearings)
    return s


def echosounder_1d(n_samples: int = 65536, seed: int = 1, n_ranges: int = 4096,
                   rmin: float = 0.5, rmax: float = 100.0, taps: int = 65) -> Workload:
    """1D EA400 38 kHz-like ping: travel ~ U[rmin, rmax], amplitude
    Rayleigh(1) * r^-2 * exp(i U[0, 2 pi)), 65-tap pulse at bin spacing."""
    c, f = 1500.0, 38.0e3
    res = float(linspace_resolution(rmin, rmax, n_ranges))
    pulse = pulse_at_bin_spacing(taps, res, f, c)
    rng = np.random.Generator(np.random.PCG64(seed))
    t = rng.uniform(rmin, rmax, n_samples)
    re, im = _rayleigh_phasor(rng, n_samples)
    re, im = re / t ** 2, im / t ** 2
    return Workload("echosounder_1d", 1, sensor_1d(rmin, rmax, n_ranges, c, pulse, taps * res),
                    _pack(re, im, t), dict(frequency=f))


def oculus_2d(n_samples: int = 1 << 20, seed: int = 2, n_bearings: int = 512, n_ranges: int = 1024,
              rmin: float = 0.3, rmax: float = 40.0, taps: int = 33, half_bearings: int = 16,
              altitude: float = 5.0, clutter: float = 0.01) -> Workload:
    """2D Oculus M1200d-like ping: 512 arcsin-spaced bearings over +/-65 deg,
    flat seafloor at 5 m altitude plus 1% volume clutter, Rayleigh amplitudes,
    33-tap pulse at bin spacing x sinc^2 beam truncated to +/-16 bearings."""
    c, f = 1500.0, 1.2e6
    res = float(linspace_resolution(rmin, rmax, n_ranges))
    bearings = arcsin_bearings(n_bearings, 130.0)
    spacing = 130.0 * DEG / (n_bearings - 1)
    span = (2 * half_bearings + 1) * spacing
    beam_taps = 8 * (2 * half_bearings + 1) + 1
    beam = beam_sinc2(beam_taps, span, 0.6 * DEG)
    pulse = pulse_at_bin_spacing(taps, res, f, c)
    rng = np.random.Generator(np.random.PCG64(seed))
    th = rng.uniform(-65.0 * DEG, 65.0 * DEG, n_samples)
    sin_dep = rng.uniform(altitude / rmax, 1.0, n_samples)
    t = altitude / sin_dep
    vol = rng.random(n_samples) < clutter
    t[vol] = rng.uniform(rmin, rmax, int(vol.sum()))
    re, im = _rayleigh_phasor(rng, n_samples)
    return Workload("oculus_2d", 2,
                    sensor_2d(rmin, rmax, n_ranges, c, pulse, taps * res, beam, span, bearings),
                    _pack(re, im, t, th), dict(frequency=f))


def precision_2d(n_samples: int = 1 << 24, seed: int = 3, n_bearings: int = 512, n_ranges: int = 4096,
                 rmin: float = 0.3, rmax: float = 120.0, taps: int = 33) -> Workload:
    """Dense-directivity 512-bearing ping at 1.2 MHz: travel ~ U[rmin, rmax],
    bearing ~ U over the fan, amplitude Rayleigh(1) * r^-2 * random phase;
    sinc^2 beam floored at -40 dB over the whole fan (every sample reaches
    every bearing), 33-tap pulse at bin spacing."""
    c, f = 1500.0, 1.2e6
    res = float(linspace_resolution(rmin, rmax, n_ranges))
    bearings = arcsin_bearings(n_bearings, 130.0)
    span = 2.0 * 131.0 * DEG
    beam_res = 0.6 * DEG
    beam_taps = int(math.ceil(span / (beam_res / 8.0))) | 1
    beam = beam_sinc2(beam_taps, span, beam_res, floor=0.01)
    pulse = pulse_at_bin_spacing(taps, res, f, c)
    rng = np.random.Generator(np.random.PCG64(seed))
    t = rng.uniform(rmin, rmax, n_samples)
    th = rng.uniform(-65.0 * DEG, 65.0 * DEG, n_samples)
    re, im = _rayleigh_phasor(rng, n_samples)
    re, im = re / t ** 2, im / t ** 2
    return Workload("precision_2d", 2,
                    sensor_2d(rmin, rmax, n_ranges, c, pulse, taps * res, beam, span, bearings),
                    _pack(re, im, t, th), dict(frequency=f))


def oculus_reference_2d(n_samples: int = 20000, seed: int = 4, n_bearings: int = 256) -> Workload:
    """The reference's own Oculus M1200d receiver parameters
    (examples/oculus_M1200d_1_receiver.yaml): ranges Linspace(0.1, 6.5, 500),
    1.2 MHz Waveform_Sine with adaptive duration and 8x oversampling, sinc
    beamsteering with 0.6 deg resolution over 130 deg, 256 arcsin bearings."""
    rmin, rmax, n_ranges, c, f = 0.1, 6.5, 500, 1500.0, 1.2e6
    duration = adaptive_duration(rmin, rmax, n_ranges, c)
    pulse = waveform_sine(f, float(duration), 8)
    span, res_b = 130.0 * DEG, 0.6 * DEG
    beam = beam_sinc(span, res_b, 8)
    bearings = arcsin_bearings(n_bearings, 130.0)
    rng = np.random.Generator(np.random.PCG64(seed))
    t = rng.uniform(0.05, 6.6, n_samples)
    th = rng.uniform(-66.0 * DEG, 66.0 * DEG, n_samples)
    re, im = _rayleigh_phasor(rng, n_samples)
    sensor = dict(range_min=rmin, range_max=rmax, range_count=n_ranges, sound_celerity=c,
                  pulse_duration=float(duration), margin=float(F32(F32(c) * duration)), pulse=pulse,
                  beam=beam, beam_span=span, bearings=bearings)
    return Workload("oculus_reference_2d", 2, sensor, _pack(re, im, t, th), dict(frequency=f))


def ea400_reference_1d(n_samples: int = 20000, seed: int = 5) -> Workload:
    """The reference's EA400 38 kHz receiver (examples/EA400_38KHz_receiver.yaml):
    ranges Linspace(0.1, 49.999, 1049), fixed 128 us Waveform_Sine, 8x
    oversampling."""
    rmin, rmax, n_ranges, c, f, duration = 0.1, 49.999, 1049, 1500.0, 38.0e3, 128.0e-6
    pulse = waveform_sine(f, duration, 8)
    rng = np.random.Generator(np.random.PCG64(seed))
    t = rng.uniform(0.0, 51.0, n_samples)
    re, im = _rayleigh_phasor(rng, n_samples)
    sensor = dict(range_min=rmin, range_max=rmax, range_count=n_ranges, sound_celerity=c,
                  pulse_duration=float(F32(duration)), margin=float(F32(F32(c) * F32(duration))), pulse=pulse)
    return Workload("ea400_reference_1d", 1, sensor, _pack(re, im, t), dict(frequency=f))


CONFIGS = {
    "echosounder_1d": echosounder_1d,
    "oculus_2d": oculus_2d,
    "precision_2d": precision_2d,
    "oculus_reference_2d": oculus_reference_2d,
    "ea400_reference_1d": ea400_reference_1d,
}
