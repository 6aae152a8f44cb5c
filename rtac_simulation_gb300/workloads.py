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


def baseband_pulse(taps: int) -> np.ndarray:
    """Gaussian pulse envelope (complex baseband, sigma = taps / 6 taps), one
    tap per range bin: the carrier is carried by each sample's phase."""
    d = np.arange(taps, dtype=np.float64) - (taps - 1) / 2.0
    return np.exp(-0.5 * (d / (taps / 6.0)) ** 2).astype(np.complex64)


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


ECHO_PHASE = 1
ECHO_SPREADING = 2

# Receive-array phase reference of the precision workload, 3 mm from the
# sensor origin along the array: the beam response then carries the phase
# exp(i kappa (sin theta_k - sin theta_b)), kappa = 2 pi x0 / lambda, and the
# dense bearing directivity is complex.
PHASE_CENTRE_M = 3.0e-3


def steering_wavenumber(frequency: float, c: float, x0: float) -> float:
    """kappa = 2 pi x0 / lambda of a phase reference x0 metres off the origin."""
    return 2.0 * math.pi * x0 * frequency / c


def steer_samples(samples: np.ndarray, steer: float) -> np.ndarray:
    """Copy of 2D samples with each value multiplied by exp(i kappa sin theta_s):
    with the output rotated by exp(-i kappa sin theta_b) (steer_ping), the
    per-sample PSF of a real beam becomes the per-sample counterpart of the
    steered complex directivity of precision_tables."""
    out = np.array(samples, dtype=np.float32, copy=True)
    if steer == 0.0:
        return out
    ph = np.exp(1j * steer * np.sin(out[:, 3].astype(np.float64)))
    v = (out[:, 0].astype(np.float64) + 1j * out[:, 1]) * ph
    out[:, 0], out[:, 1] = v.real, v.imag
    return out


def steer_ping(ping: np.ndarray, bearings, steer: float) -> np.ndarray:
    """ping[r][b] * exp(-i kappa sin theta_b) (see steer_samples)."""
    if steer == 0.0:
        return ping
    return ping * np.exp(-1j * steer * np.sin(np.asarray(bearings, np.float64)))[None, :]


@dataclass
class Workload:
    name: str
    dims: int
    sensor: dict
    samples: np.ndarray               # (N, 3) SimSample1D or (N, 4) SimSample2D, float32
    meta: dict = field(default_factory=dict)
    echo: dict | None = None          # echo pre-step: {"carrier_hz": f, "flags": ECHO_*}
    precision: dict = field(default_factory=dict)   # keyword arguments of precision_tables

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


def on_range_grid(samples: np.ndarray, sensor: dict, every: int = 8, seed: int = 99) -> np.ndarray:
    """Copy of `samples` in which every `every`-th travel is set exactly to a
    (seeded, random) output range R_r = range_min + r * resolution in float:
    with the reference's literal 1D scaling 1.0f / duration * c, only samples
    at an exact output range fall inside the pulse table, so these give that
    ping its non-zero rows."""
    out = np.array(samples, dtype=np.float32, copy=True)
    rng = np.random.Generator(np.random.PCG64(seed))
    idx = np.arange(0, out.shape[0], every)
    R = linspace(sensor["range_min"], sensor["range_max"], sensor["range_count"])
    out[idx, 2] = R[rng.integers(0, R.size, idx.size)]
    return out


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
    bearing ~ U over the fan, reflectivity Rayleigh(1) * random phase; the
    echo pre-step applies the carrier phase 4 pi f d / c (reduced in FP64)
    and the r^-2 spreading on the device. Sinc^2 beam floored at -40 dB over
    the whole fan (every sample reaches every bearing), 33-tap Gaussian
    baseband pulse envelope at bin spacing (the carrier is in the samples)."""
    c, f = 1500.0, 1.2e6
    res = float(linspace_resolution(rmin, rmax, n_ranges))
    bearings = arcsin_bearings(n_bearings, 130.0)
    span = 2.0 * 131.0 * DEG
    beam_res = 0.6 * DEG
    beam_taps = int(math.ceil(span / (beam_res / 8.0))) | 1
    beam = beam_sinc2(beam_taps, span, beam_res, floor=0.01)
    pulse = baseband_pulse(taps)
    rng = np.random.Generator(np.random.PCG64(seed))
    t = rng.uniform(rmin, rmax, n_samples)
    th = rng.uniform(-65.0 * DEG, 65.0 * DEG, n_samples)
    re, im = _rayleigh_phasor(rng, n_samples)
    return Workload("precision_2d", 2,
                    sensor_2d(rmin, rmax, n_ranges, c, pulse, taps * res, beam, span, bearings),
                    _pack(re, im, t, th), dict(frequency=f, phase_centre_m=PHASE_CENTRE_M),
                    echo=dict(carrier_hz=f, flags=ECHO_PHASE | ECHO_SPREADING),
                    precision=dict(steer=steering_wavenumber(f, c, PHASE_CENTRE_M)))


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


def stress_2d(n_samples: int = 1 << 27, seed: int = 5, n_bearings: int = 1024, n_ranges: int = 8192,
              rmin: float = 0.5, rmax: float = 100.0, taps: int = 33, half_bearings: int = 16,
              cluster_fraction: float = 0.5) -> Workload:
    """Contention stress ping: 1024 arcsin bearings x 8192 ranges, 2^27
    samples. `cluster_fraction` of them form a wreck-like target, Gaussian in
    range (sigma 0.25 m at 40 m, so ~1% of the range bins hold it) and in
    bearing (sigma 3 deg at +10 deg); the rest lie on a flat seafloor at 8 m
    altitude. Rayleigh reflectivity with the 1.2 MHz echo pre-step; 33-tap
    baseband pulse x sinc^2 beam truncated to +/-16 bearings."""
    c, f = 1500.0, 1.2e6
    bearings = arcsin_bearings(n_bearings, 130.0)
    spacing = 130.0 * DEG / (n_bearings - 1)
    span = (2 * half_bearings + 1) * spacing
    beam = beam_sinc2(8 * (2 * half_bearings + 1) + 1, span, 0.6 * DEG)
    res = float(linspace_resolution(rmin, rmax, n_ranges))
    pulse = baseband_pulse(taps)
    rng = np.random.Generator(np.random.PCG64(seed))
    nc = int(n_samples * cluster_fraction)
    out = np.empty((n_samples, 4), dtype=F32)
    # cluster
    out[:nc, 2] = rng.normal(40.0, 0.25, nc)
    out[:nc, 3] = rng.normal(10.0 * DEG, 3.0 * DEG, nc)
    # seafloor
    ns = n_samples - nc
    out[nc:, 3] = rng.uniform(-65.0 * DEG, 65.0 * DEG, ns)
    out[nc:, 2] = 8.0 / rng.uniform(8.0 / rmax, 1.0, ns)
    a = rng.rayleigh(1.0, n_samples).astype(F32)
    ph = rng.uniform(0.0, 2.0 * math.pi, n_samples).astype(F32)
    out[:, 0] = a * np.cos(ph)
    out[:, 1] = a * np.sin(ph)
    perm = rng.permutation(n_samples)
    out = out[perm]
    return Workload("stress_2d", 2, sensor_2d(rmin, rmax, n_ranges, c, pulse, taps * res, beam, span, bearings),
                    out, dict(frequency=f, cluster_fraction=cluster_fraction),
                    echo=dict(carrier_hz=f, flags=ECHO_PHASE | ECHO_SPREADING))


def batched_mix(n_pings: int = 64, seed: int = 7, log2_min: float = 14.0, log2_max: float = 22.0) -> list:
    """Batched mixed-sensor set: `n_pings` pings with log-uniform sample counts
    in [2^log2_min, 2^log2_max]; 50% 512-bearing 2D (1024 ranges over
    [0.3, 40] m), 25% 256-bearing 2D (512 ranges over [0.5, 30] m), 25% 1D
    with 2048 ranges over [0.5, 100] m; per-ping pulses of 17..65 range taps
    and beams of +/-8..32 bearings."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kinds = np.array([0] * (n_pings // 2) + [1] * (n_pings // 4) + [2] * (n_pings - n_pings // 2 - n_pings // 4))
    rng.shuffle(kinds)
    pings = []
    for i, kind in enumerate(kinds):
        n = int(round(2.0 ** rng.uniform(log2_min, log2_max)))
        taps = int(rng.integers(17, 66))
        half = int(rng.integers(8, 33))
        if kind == 0:
            wk = oculus_2d(n_samples=n, seed=1000 + i, n_bearings=512, n_ranges=1024, rmin=0.3, rmax=40.0,
                           taps=taps, half_bearings=half)
        elif kind == 1:
            wk = oculus_2d(n_samples=n, seed=1000 + i, n_bearings=256, n_ranges=512, rmin=0.5, rmax=30.0,
                           taps=taps, half_bearings=half, altitude=3.0)
        else:
            wk = echosounder_1d(n_samples=n, seed=1000 + i, n_ranges=2048, rmin=0.5, rmax=100.0, taps=taps)
        wk.name = f"batch{i}_{['2d512', '2d256', '1d2048'][kind]}"
        pings.append(wk)
    return pings


CONFIGS = {
    "echosounder_1d": echosounder_1d,
    "oculus_2d": oculus_2d,
    "precision_2d": precision_2d,
    "oculus_reference_2d": oculus_reference_2d,
    "ea400_reference_1d": ea400_reference_1d,
    "batched_mix": batched_mix,
    "stress_2d": stress_2d,
}


def _lerp(table: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Texture-equivalent lerp with border addressing, exact weights."""
    n = table.shape[0]
    fl = np.floor(x)
    ok = (fl >= -1) & (fl <= n - 1)
    i = np.where(ok, fl, 0).astype(np.int64)
    a = x - fl
    pad = np.concatenate([np.zeros(1, table.dtype), table, np.zeros(1, table.dtype)])
    lo = pad[np.clip(i + 1, 0, n + 1)]
    hi = pad[np.clip(i + 2, 0, n + 1)]
    return np.where(ok, lo * (1 - a) + hi * a, 0)


# Three-point Gauss-Legendre rule on [-1, 1]: exact for polynomials up to
# degree 5, so for the (hat function x piecewise-linear beam) products of the
# projection below.
_GL3 = ((-math.sqrt(0.6), 5.0 / 9.0), (0.0, 8.0 / 9.0), (math.sqrt(0.6), 5.0 / 9.0))


def grid_points(first: float, last: float, cells: int) -> np.ndarray:
    """Bearings of the precision form's uniform grid, in float as the device
    forms them: first + q * ((last - first) / (cells - 1))."""
    step = F32(F32(F32(last) - F32(first)) / F32(cells - 1))
    q = np.arange(cells, dtype=F32)
    return (F32(first) + (q * step).astype(F32)).astype(F32)


def project_directivity(grid: np.ndarray, bearings, beam, span: float, steer: float = 0.0) -> np.ndarray:
    """Directivity of the binned model on a bearing grid: for each output
    bearing b, the least-squares (L2) projection of its response
    beam(theta - theta_b) * exp(i steer (sin theta - sin theta_b)) onto the
    hat functions of the grid, i.e. the coefficients whose linear
    interpolation between grid bearings is closest in mean square to the
    per-sample response. The beam is the texture-equivalent lerp of the table
    (border addressing); its knots split every grid interval, and each piece
    is integrated with the three-point Gauss-Legendre rule (exact when steer
    is 0). Returns complex128 [cells][nB]."""
    g = np.asarray(grid, np.float64)
    tb = np.asarray(bearings, np.float32).astype(np.float64)
    tab = np.asarray(beam, np.float32).astype(np.float64)
    W = tab.size
    kx = float(np.float32(1.0) / np.float32(span)) * W
    cx = 0.5 * W - 0.5
    h = np.diff(g)                                        # [cells - 1]
    xa = (g[:-1, None] - tb[None, :]) * kx + cx           # texel coordinate at each interval's ends
    xb = (g[1:, None] - tb[None, :]) * kx + cx
    k0 = np.floor(xa) + 1.0                               # first knot above xa
    pieces = int(math.ceil(float(h.max()) * kx)) + 1
    f = np.zeros((g.size, tb.size), np.complex128 if steer else np.float64)
    sb = np.sin(tb)[None, :]
    for m in range(pieces + 1):
        lo = xa if m == 0 else np.minimum(k0 + (m - 1), xb)
        hi = np.minimum(k0 + m, xb)
        half = 0.5 * (hi - lo)
        if not np.any(half > 0):
            continue
        mid = 0.5 * (hi + lo)
        for node, weight in _GL3:
            x = mid + half * node
            th = tb[None, :] + (x - cx) / kx
            val = _lerp(tab, x.ravel()).reshape(x.shape)
            if steer:
                val = val * np.exp(1j * steer * (np.sin(th) - sb))
            wq = weight * half / kx * val                 # quadrature weight x response (d theta = dx / kx)
            f[:-1] += wq * (g[1:, None] - th) / h[:, None]
            f[1:] += wq * (th - g[:-1, None]) / h[:, None]
    from scipy.linalg import solve_banded
    ab = np.zeros((3, g.size))
    ab[0, 1:] = h / 6.0
    ab[2, :-1] = h / 6.0
    ab[1, :-1] += h / 3.0
    ab[1, 1:] += h / 3.0
    return solve_banded((1, 1), ab, f)


def precision_tables(sensor: dict, steer: float = 0.0, grid_count: int = 0, grid_first=None, grid_last=None) -> dict:
    """Configuration of the binned precision model, derived from a 2D sensor's
    tables as rtacx_configure_precision derives them when given NULL tables:
    a uniform grid of `grid_count` bearings (default 4 x bearing_count) from
    the first to the last table bearing, the directivity projected onto it
    (project_directivity; with steer = kappa != 0 it carries the phase of a
    phase reference off the origin and is complex), and the range taps of
    the range nodes two output bins apart, one set per output-row parity
    (range_taps). Returns the keyword arguments of
    Context.configure_precision: directivity (complex64 [grid_count][nB]),
    range_taps (complex64 [2][L]), tap_center, grid_count, grid_first,
    grid_last."""
    bear = np.asarray(sensor["bearings"], np.float32)
    nB = bear.size
    cells = int(grid_count) or 4 * nB
    first = float(bear[0]) if grid_first is None else float(np.float32(grid_first))
    last = float(bear[-1]) if grid_last is None else float(np.float32(grid_last))
    g = grid_points(first, last, cells)
    D = project_directivity(g, bear, sensor["beam"], sensor["beam_span"], steer).astype(np.complex64)
    taps, center = range_taps(sensor)
    return dict(directivity=D, range_taps=taps, tap_center=center, grid_count=cells,
                grid_first=first, grid_last=last)


RANGE_STEP = 2      # output range bins per node of the precision form's range grid
TAP_PAD = 6         # taps kept beyond the nodes the pulse reaches
SOLVE_PAD = 10      # further nodes of the truncated Gram system


def range_taps(sensor: dict):
    """Range taps of the binned model, whose range grid has one node every
    RANGE_STEP = 2 output bins (node m at range_min + m * 2 * resolution).
    For output row r = 2 m + p the pulse response P(x - R_r), seen from node
    m, is P(x - p * resolution); its least-squares (L2) projection onto the
    hat functions of the nodes gives taps[p][t], the weight of node
    m + t - center. P is the texture-equivalent lerp of the pulse table
    (border addressing). The right-hand sides integrate hat x P over each
    half of every hat, split at the pulse table's knots, with the three-point
    Gauss-Legendre rule (exact: linear x linear); the Gram system of the
    uniform hats (spacing h: h / 6, 2 h / 3, h / 6) is solved on the nodes
    the pulse reaches widened by TAP_PAD + SOLVE_PAD on each side, and the
    taps of the nodes widened by TAP_PAD are kept. Returns (taps complex64
    [2][L], index of node offset 0)."""
    nR = sensor["range_count"]
    res = float(linspace_resolution(sensor["range_min"], sensor["range_max"], nR))
    hr = float(F32(RANGE_STEP) * F32(res))
    pulse = np.asarray(sensor["pulse"], np.complex64).astype(np.complex128)
    H = pulse.size
    pscale = float(np.float32(1.0) / np.float32(np.float32(sensor["pulse_duration"]) * np.float32(sensor["sound_celerity"])))
    ky, cy = pscale * H, 0.5 * H - 0.5
    y_lo, y_hi = (-1.0 - cy) / ky, (H - cy) / ky            # P is zero outside (y_lo, y_hi)
    dmin = int(math.floor(y_lo / hr)) - 1
    dmax = int(math.ceil((y_hi + (RANGE_STEP - 1) * res) / hr)) + 1
    s0, s1 = dmin - TAP_PAD - SOLVE_PAD, dmax + TAP_PAD + SOLVE_PAD
    d = np.arange(s0, s1 + 1)
    taps = []
    for p in range(RANGE_STEP):
        off = p * res
        f = np.zeros(d.size, np.complex128)
        for i, dd in enumerate(d):
            for a, b, up in (((dd - 1) * hr, dd * hr, True), (dd * hr, (dd + 1) * hr, False)):
                # knots of P(x - off) inside (a, b)
                k_lo = math.ceil((a - off) * ky + cy)
                k_hi = math.floor((b - off) * ky + cy)
                pts = [a] + [off + (k - cy) / ky for k in range(k_lo, k_hi + 1)] + [b]
                pts = sorted(x for x in pts if a <= x <= b)
                for lo, hi in zip(pts[:-1], pts[1:]):
                    half = 0.5 * (hi - lo)
                    if not half > 0:
                        continue
                    mid = 0.5 * (hi + lo)
                    for node, weight in _GL3:
                        x = mid + half * node
                        xt = np.array([(x - off) * ky + cy])
                        pv = (_lerp(pulse.real, xt) + 1j * _lerp(pulse.imag, xt))[0]
                        lam = (x - a) / hr if up else (b - x) / hr
                        f[i] += weight * half * lam * pv
        from scipy.linalg import solve_banded
        ab = np.zeros((3, d.size))
        ab[0, 1:] = hr / 6.0
        ab[1, :] = 2.0 * hr / 3.0
        ab[2, :-1] = hr / 6.0
        t = solve_banded((1, 1), ab, f)
        keep = (d >= dmin - TAP_PAD) & (d <= dmax + TAP_PAD)
        taps.append(t[keep])
    return np.array(taps, np.complex64), int(TAP_PAD - dmin)