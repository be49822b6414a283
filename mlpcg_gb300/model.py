"""BaseModel: parameter initialisation shared by all blocks (model.py:12-29 of the reference)."""
from __future__ import annotations

import math

import torch.nn as nn


class BaseModel(nn.Module):
    def __init__(self):
        super().__init__()

    def move_to(self, device):
        self.device = device
        self.to(device)

    def eval_forward(self, *args, **kwargs):
        return self.forward(*args, **kwargs)

    def reset_parameters(self, weight, bias):
        """kaiming_uniform(a=sqrt(5)) on the weight, U(-1/sqrt(fan_in), 1/sqrt(fan_in)) on the bias."""
        nn.init.kaiming_uniform_(weight, a=math.sqrt(5))
        if bias is not None:
            fan_in, _ = nn.init._calculate_fan_in_and_fan_out(weight)
            if fan_in != 0:
                bound = 1 / math.sqrt(fan_in)
                nn.init.uniform_(bias, -bound, bound)
