"""Quantum convolution layer: qandle's QConv (qandle/convolution.py:9-61) on
the batched engine.

A QConv slides a k x k window over a [batch, c_in, H, W] image.  Each window
position gives one patch of c_in * k * k values; the patch is the amplitude
vector of a small circuit (zero-padded to 2^q amplitudes, not normalised,
shifted by a small constant so that no patch is all zero), the circuit
applies one strongly entangling block, and the first c_out joint
probabilities, scaled by c_out / 2, are the output channels at that
position.

Here every patch of every image of a call becomes one sample of ONE batched
circuit run: for a 17 x 18 image in batches of 10 that is 3060 samples of a
5-qubit circuit in a single fused forward (AmplitudeEmbedding writes the
patches as the input states), instead of one small circuit per patch.  The
patch gather is torch's unfold; everything after it is a view, a slice and a
scale.  What a user sees (class, constructor, attributes, checkpoint keys,
output values and shape) is the reference's.
"""
from __future__ import annotations

import math
import typing

import torch

from . import ansaetze, embeddings, measurements, qcircuit

__all__ = ["QConv"]

# Added to every patch value before embedding, so that an all-zero patch
# (padding, black image regions) still has a norm (the reference's value).
PATCH_SHIFT = 0.001


def _pair(v) -> typing.Tuple[int, int]:
    return tuple(v) if isinstance(v, (tuple, list)) else (v, v)


class QConv(torch.nn.Module):
    def __init__(self, in_channels: int, out_channels: int,
                 kernel_size: typing.Union[typing.Tuple[int, int], int] = (3, 3),
                 padding: typing.Union[typing.Tuple[int, int], int] = (1, 1), qdepth: int = 1,
                 **engine_options):
        super().__init__()
        self.in_channels = in_channels
        self.out_channels = out_channels
        self.qdepth = qdepth
        self.kernel_size = _pair(kernel_size)
        self.padding = _pair(padding)
        kh, kw = self.kernel_size
        # enough qubits for a whole patch and for the output channels
        self.qubits = max(math.ceil(math.log2(kh * kw * in_channels)), math.ceil(math.log2(out_channels)), 1)
        wires = list(range(self.qubits))
        self.unfold = torch.nn.Unfold(kernel_size=kernel_size, padding=self.padding)
        self.qcircuit = qcircuit.Circuit(
            num_qubits=self.qubits,
            layers=[embeddings.AmplitudeEmbedding(qubits=wires, pad_with=0, name="emb"),
                    ansaetze.StronglyEntanglingLayer(qubits=wires, depth=self.qdepth),
                    measurements.MeasureJointProbability()],
            **engine_options)

    def output_size(self, h: int, w: int) -> typing.Tuple[int, int]:
        """Spatial size of the output (stride 1, the layer's padding)."""
        (kh, kw), (ph, pw) = self.kernel_size, self.padding
        return h + 2 * ph - kh + 1, w + 2 * pw - kw + 1

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        if x.dim() != 4:
            raise ValueError(f"QConv takes [batch, channels, height, width] inputs, got shape {tuple(x.shape)}")
        b, c, h, w = x.shape
        if c != self.in_channels:
            raise ValueError(f"Input channels {c} does not match in_channels {self.in_channels}")
        ho, wo = self.output_size(h, w)
        patches = self.unfold(x)                                  # [b, c*kh*kw, ho*wo]
        states_in = patches.transpose(1, 2).reshape(b * ho * wo, -1) + PATCH_SHIFT
        probs = self.qcircuit(emb=states_in)                      # [b*ho*wo, 2^qubits], one batched run
        y = probs[:, :self.out_channels] * (self.out_channels / 2)
        return y.reshape(b, ho, wo, self.out_channels).permute(0, 3, 1, 2)
