"""Helpers shared by the GPU tests: device round trips through the C ABI."""
import numpy as np


def padded(x, dtype=np.float64):
    nx, ny = x.shape
    out = np.zeros((nx, 2 * (ny // 2 + 1)), dtype=dtype)
    out[:, :ny] = x
    return out


def to_complex(p):
    p = np.ascontiguousarray(p)
    return p.view(np.complex128 if p.dtype == np.float64 else np.complex64)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    d = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (d if d else 1.0))


def run_device(torch, plan, host, op="forward"):
    """Copy `host` (padded layout, any leading batch dims) to the GPU, run `op`
    on the plan's stream set to torch's current stream, copy back."""
    dev = torch.from_numpy(np.ascontiguousarray(host)).cuda()
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    ptr = dev.data_ptr()
    if op == "forward":
        plan.execute_device(ptr)
    elif op == "backward":
        plan.backward_device(ptr)
    elif op == "c2r":
        plan.c2r_device(ptr)
    else:
        raise ValueError(op)
    torch.cuda.synchronize()
    out = dev.cpu().numpy()
    plan.set_stream(None)
    return out
