"""The upload buffer pool (host logic; CPU tensors stand in for device ones)."""
import threading

import torch

from snapatac2_gb300.tools import _UploadPool


def test_pool_reuses_and_grows():
    p = _UploadPool()
    dev = torch.device("cpu")
    a = p.take(dev, torch.int32, 100)
    assert a.numel() >= 100
    p.give(a)
    b = p.take(dev, torch.int32, 50)          # reused (large enough)
    assert b.data_ptr() == a.data_ptr()
    c = p.take(dev, torch.int32, 10)          # pool empty while b is lent: fresh buffer
    assert c.data_ptr() != b.data_ptr()
    p.give(b)
    p.give(c)                                 # the larger of the two stays
    assert p.pooled_bytes() == a.numel() * 4
    d = p.take(dev, torch.int32, 1000)        # too small: grown
    assert d.numel() >= 1000
    p.give(d)
    assert p.pooled_bytes() == d.numel() * 4
    assert p.take(dev, torch.float64, 8).dtype == torch.float64   # keyed by dtype
    p.clear()
    assert p.pooled_bytes() == 0


def test_pool_threads_never_share_a_buffer():
    p = _UploadPool()
    dev = torch.device("cpu")
    held, lock = [], threading.Lock()

    def worker():
        for _ in range(200):
            b = p.take(dev, torch.uint8, 64)
            with lock:
                assert all(b.data_ptr() != h for h in held)
                held.append(b.data_ptr())
            with lock:
                held.remove(b.data_ptr())
            p.give(b)

    ts = [threading.Thread(target=worker) for _ in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
