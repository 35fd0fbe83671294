"""Angle remapping functions applied to trainable angles before t = theta / 2.

The reference takes them from the third-party ``qw_map`` package
(qw-map 0.1.2; qandle/config.py:1-3, operators.py:168-171, :271).  That
package is not a dependency here.  ``none`` is the identity the reference
uses for ``remapping=None``; ``tanh`` restates qw_map's published tanh
mapping, pi * tanh(x).  Only ``none`` is pinned by parity tests.

Any callable on tensors works as a remapping: the engine evaluates it with
torch on the device and differentiates through it with torch autograd.
"""
import math

import torch


def none(x):
    return x


def tanh(x):
    return torch.tanh(x) * math.pi
