"""FP64 training pass in torch (float64 on whichever device the tensors live):
the check that a long GPU training run is compared against. Test
infrastructure only.

It restates, without any 16-bit rounding, what the reference trains
(shader/src/nrc_gradient.comp:26-58 with NN_nv.glsl): the 64-wide MLP with five
ReLU layers and a 3-output layer (weights row-major W[out][in], y = W x), the
relative-L2 luminance loss gradient 2 (p - t) / (lum(max(p, 0))^2 + 0.01) with
the denominator held constant (NN_nv.glsl:178-196) on the unclamped output,
ReLU backward masked by the layer input being > 0, weight gradients summed over
the batch and divided by the record count, and Adam with bias correction
(nrc_optimize.comp:32-54). The per-record loss it reports is
sum_c (p_c - t_c)^2 / (lum^2 + 0.01) at the weights before the step, as the
GPU's FP64 check-path accumulator reports it. tests/test_fp64_pass.py checks it
against the C oracle's FP64 mode (oracle_train_grad_w64).
"""
import torch

P = 20672
LUM = (0.299, 0.587, 0.114)


def split(w):
    """Views of the parameter vector: five 64x64 hidden layers and the 3x64 output layer."""
    return [w[l * 4096:(l + 1) * 4096].view(64, 64) for l in range(5)] + [w[20480:].view(3, 64)]


def grad_and_loss(w, x, t):
    """Sum over the batch of the weight gradient, and of the per-record loss.
    w: (P,) float64; x: (n, 64) float64 features; t: (n, 3) float64 targets."""
    W = split(w)
    acts = [x]
    a = x
    for l in range(5):
        a = torch.relu(a @ W[l].T)
        acts.append(a)
    p = a @ W[5].T
    lum = torch.relu(p) @ torch.tensor(LUM, dtype=p.dtype, device=p.device)
    den = (lum * lum + 0.01)[:, None]
    loss = ((p - t) ** 2 / den).sum()
    g = 2.0 * (p - t) / den
    grads = [None] * 6
    for l in range(5, -1, -1):
        grads[l] = g.T @ acts[l]
        if l > 0:
            g = (g @ W[l]) * (acts[l] > 0)
    return torch.cat([gl.reshape(-1) for gl in grads]), loss


class Fp64Adam:
    """FP64 weights and moments; Adam as nrc_optimize.comp without fp16 rounding."""

    def __init__(self, w32, lr, beta1, beta2, eps, device):
        self.w = torch.as_tensor(w32, device=device).double().clone()
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.lr, self.b1, self.b2, self.eps = lr, beta1, beta2, eps
        self.b1t = self.b2t = 1.0

    def step(self, x, t):
        """One training step on a batch; returns the batch's mean loss before the update."""
        n = x.shape[0]
        g, loss = grad_and_loss(self.w, x, t)
        g = g / n
        self.b1t *= self.b1
        self.b2t *= self.b2
        self.m.mul_(self.b1).add_((1.0 - self.b1) * g)
        self.v.mul_(self.b2).add_((1.0 - self.b2) * g * g)
        self.w -= self.lr * (self.m / (1.0 - self.b1t)) / (torch.sqrt(self.v / (1.0 - self.b2t)) + self.eps)
        return loss / n
