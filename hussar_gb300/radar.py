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
        """radar.h:534-546: grid index (chirp, sample, channel) of the largest magnitude."""
        i = int(np.argmax(np.abs(self.data.reshape(-1))))
        return np.unravel_index(i, self.data.shape)

    def tobytes(self):
        """Raw complex64 in [chirp][sample][channel] order, as writeFrameToFile writes it
        (examples/src/utils.h:29-35)."""
        return self.data.astype(np.complex64).tobytes()
