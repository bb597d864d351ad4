"""Helpers shared by the GPU tests."""
import numpy as np
import torch


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def count(n: int) -> torch.Tensor:
    return torch.tensor([n], dtype=torch.int32, device="cuda")


def host(t: torch.Tensor) -> np.ndarray:
    torch.cuda.synchronize()
    return t.cpu().numpy()


def f16(u16: np.ndarray) -> np.ndarray:
    return u16.view(np.float16).astype(np.float64)
