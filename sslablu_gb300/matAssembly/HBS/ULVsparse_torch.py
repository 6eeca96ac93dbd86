"""ULV factorisation and solve of HBS matrices in block-tensor form -- drop-in
for the public functions of SslabLU matAssembly/HBS/ULVsparse_torch.py.

    convert_to_torch_tens(A, Nb, device)    (Nb*n, k) -> (Nb, n, k)   (14-20)
    convert_to_blkdiag(A)                   (Nb, n, k) -> (Nb*n, k)   (21-28)
    compute_ULV(Utens, Dtens, Vtens, Nbvec, device)
        -> Qlist, Wlist, Uulist, Rlist, NNvec                         (231-295)
    solve(Umats, Dmats, Qlist, Wlist, Uulist, Rlist, NNvec, rhs, device,
          mode='N')                                                   (297-363)

Factors are lists of (Nb, n, k) tensors, leaves first (the layout of
HBStorch.HBSMAT).  The arithmetic is ULVsparse's (the torch module batches
the same per-block QR and block products); it runs in libslablu through the
ULVsparse drop-in, and results come back as float64 tensors on ``device``
(CUDA when None or not a torch device).  The right-hand side is in tree (block) order.
"""
import numpy as np
import torch

from . import ULVsparse as _ulv


def _dev(device):
    """Where results go: the given torch device, else the GPU (upstream's
    assembler passes a device *name*, which is not a torch device)."""
    if device is None:
        return "cuda"
    try:
        return torch.device(device)
    except (RuntimeError, TypeError):
        return "cuda"


def convert_to_torch_tens(A, Nb, device):
    A = torch.as_tensor(A, dtype=torch.float64)
    n = A.shape[0] // Nb
    return A.reshape(Nb, n, A.shape[1]).to(device if device is not None else A.device)


def convert_to_blkdiag(A):
    A = torch.as_tensor(A)
    return A.reshape(A.shape[0] * A.shape[1], A.shape[2])


def _flat(T):
    return torch.as_tensor(T, dtype=torch.float64).reshape(-1, T.shape[-1]).to("cuda")


def _blocks(M, Nb, device):
    M = torch.as_tensor(np.ascontiguousarray(M)) if not isinstance(M, torch.Tensor) else M
    return M.reshape(Nb, M.shape[0] // Nb, M.shape[1]).to(device)


def compute_ULV(Utens, Dtens, Vtens, Nbvec, device):
    """ULVsparse_torch.py:231-295."""
    Nb = [int(D.shape[0]) for D in Dtens]
    Q, W, Uu, R, NN = _ulv.compute_ULV([_flat(U) for U in Utens], [_flat(D) for D in Dtens],
                                       [_flat(V) for V in Vtens], Nb)
    dv = _dev(device)
    Lv = len(Dtens)
    return ([_blocks(Q[t], Nb[t], dv) for t in range(Lv)],
            [_blocks(W[t], Nb[t], dv) for t in range(Lv - 1)],
            [_blocks(Uu[t], Nb[t], dv) for t in range(Lv - 1)],
            [_blocks(R[t], Nb[t], dv) for t in range(Lv)],
            [int(x) for x in NN])


def solve(Umats, Dmats, Qlist, Wlist, Uulist, Rlist, NNvec, rhs, device, mode="N"):
    """ULVsparse_torch.py:297-363."""
    if mode not in ("N", "T"):
        raise NotImplementedError("mode not recognized")
    Nb = [int(D.shape[0]) for D in Dmats]
    one = rhs.ndim == 1
    b = torch.as_tensor(rhs, dtype=torch.float64).to("cuda")
    x = _ulv.solve([_flat(U) for U in Umats], [_flat(D) for D in Dmats],
                   [_flat(Q) for Q in Qlist], [_flat(W) for W in Wlist],
                   [_flat(U) for U in Uulist], [_flat(R) for R in Rlist], NNvec, Nb,
                   b[:, None] if one else b, mode=mode)
    x = x[:, 0] if one else x
    return x.to(_dev(device))
