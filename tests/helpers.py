"""Device-buffer plumbing for the GPU tests (torch tensors as raw buffers)."""
import numpy as np


def dev(torch, a):
    """numpy array -> CUDA tensor with the same bytes."""
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.copy()).cuda()


def empty(torch, n, dtype):
    return torch.empty(int(max(n, 1)), dtype=dtype, device="cuda")


def ptr(t):
    return t.data_ptr()


def host(t, n=None):
    a = t.cpu().numpy()
    return a if n is None else a[:n]


def stream(torch):
    return torch.cuda.current_stream().cuda_stream


def bits_to_bytes(words, P):
    """Bit-packed particle masks (uint32 words, LSB first) -> one byte per particle."""
    w = np.ascontiguousarray(words).view(np.uint32).reshape(-1, (P + 31) // 32)
    b = np.unpackbits(w.view(np.uint8).reshape(w.shape[0], -1), axis=1, bitorder="little")
    return b[:, :P].astype(np.uint8)
