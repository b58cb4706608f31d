"""TopOptUNet: the 3-D U-Net of src/am/ai/model.py:18-67 (in_channels 4 -- design
mask and load x, y, z --, out_channels 1 -- density --, features (32, 64, 128,
256)), implemented by the engine (am_unet_* in include/am_gpu.h): BF16
convolutions with FP32 accumulate on the tensor cores, a sigmoid output."""
from __future__ import annotations

import os
from typing import Tuple

import numpy as np

from .. import _native as nat


def _pad8(v: int) -> int:
    return (int(v) + 7) // 8 * 8


class TopOptUNet:
    """3-D U-Net for topology-optimisation density prediction.

    Input (C, D, H, W), output density (D, H, W) in [0, 1].  Each of the four
    levels doubles the width; ``features`` must be (f, 2f, 4f, 8f) with f 16 or 32."""

    def __init__(self, in_channels: int = 4, out_channels: int = 1,
                 features: Tuple[int, ...] = (32, 64, 128, 256), seed: int = 0):
        features = tuple(int(f) for f in features)
        f0 = features[0]
        if len(features) != 4 or features != (f0, 2 * f0, 4 * f0, 8 * f0) or f0 not in (16, 32):
            raise ValueError("features must be (f, 2f, 4f, 8f) with f = 16 or 32")
        self.in_channels = int(in_channels)
        self.out_channels = int(out_channels)
        self.features = features
        self.net = nat.UNet(self.in_channels, self.out_channels, f0, seed)
        self.meta = {}

    def forward(self, x: np.ndarray) -> np.ndarray:
        """x: (N, C, D, H, W) with D, H, W multiples of 8 -> sigmoid outputs (N, out, D, H, W)."""
        x = np.asarray(x, dtype=np.float32)
        y = self.net.forward(np.moveaxis(x, 1, -1), sigmoid=True)
        return np.moveaxis(y, -1, 1)

    def predict(self, domain_tensor: np.ndarray) -> np.ndarray:
        """Density field (D, H, W) from an input encoding (C, D, H, W) of any size
        (zero-padded to multiples of 8 for the network)."""
        t = np.asarray(domain_tensor, dtype=np.float32)
        C, D, H, W = t.shape
        if C != self.in_channels:
            raise ValueError(f"expected {self.in_channels} input channels, got {C}")
        x = np.zeros((1, _pad8(D), _pad8(H), _pad8(W), C), np.float32)
        x[0, :D, :H, :W] = np.moveaxis(t, 0, -1)
        return self.net.forward(x, sigmoid=True)[0, :D, :H, :W, 0]

    def save(self, path: str) -> None:
        """Weights (FP32) and the architecture, in a .npz file."""
        np.savez_compressed(path, weights=self.net.get_params(), in_channels=self.in_channels,
                            out_channels=self.out_channels, features=np.array(self.features),
                            **{f"meta_{k}": np.asarray(v) for k, v in self.meta.items()})


def load_pretrained(checkpoint_path: str) -> TopOptUNet:
    """A TopOptUNet with the architecture and weights of a checkpoint written by
    TopOptUNet.save (model.py:70-82 of the reference names this entry point)."""
    if not os.path.exists(checkpoint_path):
        raise FileNotFoundError(checkpoint_path)
    d = np.load(checkpoint_path)
    m = TopOptUNet(int(d["in_channels"]), int(d["out_channels"]), tuple(int(f) for f in d["features"]))
    m.net.set_params(d["weights"])
    m.meta = {k[5:]: d[k].item() if d[k].ndim == 0 else d[k] for k in d.files if k.startswith("meta_")}
    return m
