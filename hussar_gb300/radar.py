"""libradar's FMCW types (libradar/include/radar/radar.h): RFConfig, FrameConfig and the
radar cube Frame, with the same field names and meaning.
"""
import dataclasses

import numpy as np

from . import _lib

SPEED_OF_LIGHT = np.float32(299792458.0)  # radar.h:107 (stored as float)


@dataclasses.dataclass
class RFConfig:
    """radar::RFConfig (radar.h:113-136). Units: Hz, Hz/s, Hz, s, s, s."""
    startFreq: float = 0.0
    freqSlope: float = 0.0
    adcRate: float = 0.0
    idleTime: float = 0.0
    rampTime: float = 0.0
    antennaDelay: float = 0.0

    def bandwidth(self):
        """radar.h:128-130: freqSlope * rampTime (in float, as the reference)."""
        return float(np.float32(self.freqSlope) * np.float32(self.rampTime))

    def chirpFrequency(self):
        """radar.h:133-135."""
        return float(np.float32(1.0) / (np.float32(self.idleTime) + np.float32(self.rampTime)))

    def to_c(self):
        return _lib.RFConfigC(*(np.float32(getattr(self, f.name)) for f in dataclasses.fields(self)))


@dataclasses.dataclass
class FrameConfig:
    """radar::FrameConfig (radar.h:141-164)."""
    chirpCount: int = 1
    samplesPerChirp: int = 1
    channelCount: int = 1

    def sampleCount(self):
        return int(self.chirpCount) * int(self.samplesPerChirp) * int(self.channelCount)

    def to_c(self):
        return _lib.FrameConfigC(self.chirpCount, self.samplesPerChirp, self.channelCount)


class Frame:
    """radar::Frame (radar.h:173-701): a complex64 radar cube [chirp][sample][channel].

    data is a numpy complex64 array of shape (chirpCount, samplesPerChirp, channelCount).
    """

    def __init__(self, config=None):
        self._config = FrameConfig()
        self.data = np.zeros((1, 1, 1), np.complex64)
        if config is not None:
            self.configure(config)

    def configure(self, config):
        """radar.h:347-359 (the data is zeroed here rather than left undefined)."""
        self._config = FrameConfig(config.chirpCount, config.samplesPerChirp, config.channelCount)
        self.data = np.zeros((config.chirpCount, config.samplesPerChirp, config.channelCount), np.complex64)

    def config(self):
        return FrameConfig(self._config.chirpCount, self._config.samplesPerChirp, self._config.channelCount)

    def clear(self):
        """radar.h:339-341."""
        self.data[...] = 0

    def sampleCount(self):
        return self._config.sampleCount()

    def __call__(self, i):
        """Element i of the flattened cube (radar.h:453-455, makeIndex order)."""
        return self.data.reshape(-1)[i]

    def __truediv__(self, f):
        """radar.h:388-392: a copy scaled by 1.f / f (single precision)."""
        out = Frame(self._config)
        inv = np.float32(1.0) / np.float32(f)
        out.data = (self.data.view(np.float32) * inv).view(np.complex64).reshape(self.data.shape)
        return out

    def __iadd__(self, other):
        self.data += other.data
        return self

    def argmax(self):
        """radar.h:534-546: grid index (chirp, sample, channel) of the first element with
        the largest magnitude, the magnitude evaluated as std::abs(radar::complex) does
        in single precision (complex.h:225-237: s * sqrt((x/s)^2 + (y/s)^2), s = max|.|)."""
        i = int(np.argmax(complex_abs(self.data.reshape(-1))))
        return np.unravel_index(i, self.data.shape)

    def fft(self):
        """radar.h:412-435: in-place forward 3-D DFT of the cube (FFTW_FORWARD, unnormalised,
        over chirps, samples and channels). Evaluated in FP64 and rounded to complex64
        (the reference uses FFTW in single precision)."""
        self.data = np.fft.fftn(self.data.astype(np.complex128), axes=(0, 1, 2)).astype(np.complex64)

    def tobytes(self):
        """Raw complex64 in [chirp][sample][channel] order, as writeFrameToFile writes it
        (examples/src/utils.h:29-35)."""
        return self.data.astype(np.complex64).tobytes()


def complex_abs(z):
    """std::abs(radar::complex<float>) (libradar/include/radar/complex.h:225-237),
    elementwise in float32: the larger component scales both before the square root."""
    z = np.asarray(z, np.complex64)
    x = np.abs(z.real).astype(np.float32)
    y = np.abs(z.imag).astype(np.float32)
    s = np.maximum(x, y)
    out = np.zeros(z.shape, np.float32)
    nz = s != 0
    xs = x[nz] / s[nz]
    ys = y[nz] / s[nz]
    out[nz] = s[nz] * np.sqrt(xs * xs + ys * ys)
    return out
