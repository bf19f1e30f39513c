"""Range noise with rmagine's interface (noise/Noise.hpp, GaussianNoise.hpp, RelGaussianNoise.hpp,
UniformDustNoise.hpp and their CUDA twins), computing on the GB300 through rmg_noise_apply.

    noise = GaussianNoise(0.0, 0.02, NoiseOptions(seed=42))
    noise.apply(bundle.ranges)        # device float32 tensor, in place

Each apply draws fresh numbers (the object's call counter advances); the numbers are a pure
function of (seed, call, element), so two objects with the same seed repeat each other.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib as L


@dataclass
class NoiseOptions:
    """Noise::Options (noise/Noise.hpp:53-56)."""
    seed: int = 42
    max_range: float = 10000.0


class _Noise:
    kind = -1

    def __init__(self, options: NoiseOptions | None = None):
        self.options = options or NoiseOptions()
        self.call = 0

    def _params(self) -> L.NoiseC:
        p = L.NoiseC()
        p.kind = self.kind
        p.max_range = float(self.options.max_range)
        p.seed = int(self.options.seed) & 0xFFFFFFFFFFFFFFFF
        p.call = self.call
        return p

    def _fill(self, p: L.NoiseC) -> None:
        raise NotImplementedError

    def apply(self, ranges: torch.Tensor) -> torch.Tensor:
        """Adds noise to a float32 CUDA tensor of ranges in place (asynchronous, current stream)."""
        if not (isinstance(ranges, torch.Tensor) and ranges.is_cuda and ranges.dtype == torch.float32
                and ranges.is_contiguous()):
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "noise.apply", "ranges must be a contiguous float32 CUDA tensor")
        p = self._params()
        self._fill(p)
        L.call("rmg_noise_apply", C.byref(p), C.c_void_p(ranges.data_ptr()), ranges.numel(),
               C.c_void_p(torch.cuda.current_stream().cuda_stream))
        self.call += 1
        return ranges


def device_status(clear: bool = False) -> int:
    """The noise kernels' device error word (0, or RMG_ERR_TIMEOUT after a lost bulk copy);
    synchronises the device."""
    v = C.c_uint32(0)
    L.call("rmg_noise_status", C.byref(v), 1 if clear else 0)
    return int(v.value)


class GaussianNoise(_Noise):
    """GaussianNoiseCuda: r += N(0, 1) * stddev + mean for r <= max_range."""
    kind = L.RMG_NOISE_GAUSSIAN

    def __init__(self, mean: float, stddev: float, options: NoiseOptions | None = None):
        super().__init__(options)
        self.mean, self.stddev = float(mean), float(stddev)

    def _fill(self, p):
        p.mean, p.stddev = self.mean, self.stddev


class RelGaussianNoise(_Noise):
    """RelGaussianNoiseCuda: r += N(0, 1) * stddev * r^range_exp + mean for r <= max_range."""
    kind = L.RMG_NOISE_REL_GAUSSIAN

    def __init__(self, mean: float, stddev: float, range_exp: float, options: NoiseOptions | None = None):
        super().__init__(options)
        self.mean, self.stddev, self.range_exp = float(mean), float(stddev), float(range_exp)

    def _fill(self, p):
        p.mean, p.stddev, p.range_exp = self.mean, self.stddev, self.range_exp


class UniformDustNoise(_Noise):
    """UniformDustNoiseCuda: early returns from dust with hit / return probabilities per metre."""
    kind = L.RMG_NOISE_UNIFORM_DUST

    def __init__(self, hit_probability: float, return_probability: float, options: NoiseOptions | None = None):
        super().__init__(options)
        self.hit_probability, self.return_probability = float(hit_probability), float(return_probability)

    def _fill(self, p):
        p.hit_probability, p.return_probability = self.hit_probability, self.return_probability


def philox_blocks(n_blocks: int, seed: int, call: int = 0) -> torch.Tensor:
    """The generator's raw output on the device: [n_blocks, 4] uint32 bit patterns (int32 tensor)."""
    out = torch.empty((n_blocks, 4), dtype=torch.int32, device="cuda")
    p = L.NoiseC()
    p.seed, p.call = seed, call
    L.call("rmg_noise_philox", C.byref(p), C.c_void_p(out.data_ptr()), n_blocks,
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return out
