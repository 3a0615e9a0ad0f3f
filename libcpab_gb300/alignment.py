"""CpabAligner: align data by optimising a CPAB transformation
(libcpab/alignment.py).

alignment_by_sampling and alignment_by_gradient keep the reference's
signatures and algorithms (random-walk acceptance; Adam on theta with loss
norm(transform_data(x1, theta) - x2), theta starting at identity(1, 1e-6)).

alignment_by_gradient(graph=True) captures one iteration (forward, loss,
backward, Adam step) in a CUDA graph and replays it maxiter times: the losses
are written to a device tensor and read once at the end, where the reference
reads the loss back after every iteration.  The replayed iterations compute
what the eager loop computes (tested).
"""
from __future__ import annotations

import torch

from . import functions as backend
from .cpab import Cpab


class CpabAligner(object):
    """Gradient and sampling based alignment (libcpab/alignment.py:12-120)."""

    def __init__(self, cpab_class):
        assert isinstance(cpab_class, Cpab), '''The input class
            needs to be an instance of the core cpab class '''
        self.T = cpab_class
        self.backend = backend
        self.losses = None

    def alignment_by_sampling(self, x1, x2, maxiter=100):
        """Random-walk minimisation (libcpab/alignment.py:32-55)."""
        self.T._check_type(x1)
        self.T._check_type(x2)
        assert x1.shape == x2.shape, ' Two data points does not have the same shape '
        outsize = (x2.shape[2], x2.shape[3])
        current_sample = self.T.identity(1)
        current_error = self.backend.norm(x1 - x2)
        accept_ratio = 0
        for _ in range(maxiter):
            theta = 1e-1 * self.T.sample_transformation(1, mean=current_sample.flatten())
            x1_trans = self.T.transform_data(x1, theta, outsize=outsize)
            new_error = self.backend.norm(x1_trans - x2)
            if new_error < current_error:
                current_sample = theta
                current_error = new_error
                accept_ratio += 1
        print('Acceptence ratio: ', accept_ratio / maxiter * 100, '%')
        return current_sample

    def alignment_by_gradient(self, x1, x2, maxiter=100, lr=1e-2, graph=False):
        """Adam on theta (libcpab/alignment.py:58-87).  The per-iteration
        losses are kept in self.losses (a device tensor)."""
        self.T._check_type(x1)
        self.T._check_type(x2)
        assert x1.shape == x2.shape, ' Two data points does not have the same shape '
        outsize = x1.shape[2:]
        theta = self.T.identity(1, epsilon=1e-6).clone().requires_grad_(True)
        optimizer = torch.optim.Adam([theta], lr=lr, capturable=graph)
        losses = torch.zeros(maxiter, device=x1.device)

        def iteration():
            x1_trans = self.T.transform_data(x1, theta, outsize=outsize)
            loss = self.backend.norm(x1_trans - x2)
            loss.backward()
            optimizer.step()
            return loss

        if not graph:
            for i in range(maxiter):
                optimizer.zero_grad()
                losses[i] = iteration().detach()
            self.losses = losses
            return theta

        # warm up on a side stream, then restore theta and the optimiser state
        theta0 = theta.detach().clone()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(2):
                optimizer.zero_grad(set_to_none=True)
                iteration()
        torch.cuda.current_stream().wait_stream(side)
        with torch.no_grad():
            theta.copy_(theta0)
            for st in optimizer.state.values():
                for v in st.values():
                    if torch.is_tensor(v):
                        v.zero_()
        optimizer.zero_grad(set_to_none=True)
        counter = torch.zeros(1, dtype=torch.long, device=x1.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            loss = iteration()
            losses.index_copy_(0, counter, loss.detach().reshape(1))
            counter.add_(1)
        for _ in range(maxiter):
            g.replay()
        self.losses = losses
        return theta
