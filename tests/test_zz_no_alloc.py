"""The neighbour search that allocates no device memory.

wf_find_neighbors_static() runs the cuNSearch-rule search with its
temporaries in a fixed device array inside the library, for callers that
cannot call cudaMalloc.  Its lists must equal those of the domain's own
search (wf_find_neighbors + wf_get_neighbors) bit for bit, on consecutive
calls that share that array.  The caller's buffers here are torch tensors on
the GPU; torch is only the allocator of the test.
"""
import ctypes as C

import numpy as np
import pytest

from weldformgpu_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

NB = 70
MAX_PARTICLES = 65536


def _entry():
    from weldformgpu_gb300.domain import lib
    f = lib().wf_find_neighbors_static
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_char_p, C.c_int64]
    return f


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def static_lists(x, h, fill=-7):
    """Calls the entry point with caller-owned device buffers; returns host copies."""
    torch = _torch()
    dev = torch.device("cuda:0")
    n = len(x)
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64).reshape(-1)).to(dev)
    cd = torch.full((n,), fill, dtype=torch.int32, device=dev)
    ld = torch.full((n, NB), fill, dtype=torch.int32, device=dev)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = _entry()(xd.data_ptr(), n, h, cd.data_ptr(), ld.data_ptr(), stream, err, 256)
    assert rc == 0, err.value.decode()
    return cd.cpu().numpy(), ld.cpu().numpy()


def domain_lists(x, h):
    from weldformgpu_gb300 import Domain_d
    dom = Domain_d(len(x))
    try:
        dom.set_h(h)
        dom.set_positions(x)
        dom.find_neighbors()
        return dom.get_neighbors()
    finally:
        dom.close()


def assert_same(static, domain, fill=-7):
    (cs, ls), (cd, ld) = static, domain
    assert np.array_equal(cs, cd)
    used = np.arange(NB)[None, :] < cd[:, None]
    assert np.array_equal(ls[used], ld[used])
    assert np.all(ls[~used] == fill)        # nothing written past each count


def _cases():
    # 19,488 jittered-lattice particles (grid of ~4,900 cells), then 5,244
    # reference-generator particles (~2,200 cells)
    big = S.compression_cylinder(R=0.008, H=0.012, generator="lattice", jitter=0.01, seed=7)
    small = S.compression_cylinder(R=0.005, H=0.010)
    return big, small


def test_static_search_matches_domain_search_on_consecutive_calls():
    big, small = _cases()
    assert big["n"] > small["n"]            # the second call leaves a larger grid behind
    s1 = static_lists(big["x"], big["h"])
    s2 = static_lists(small["x"], small["h"])
    s3 = static_lists(big["x"], big["h"])
    assert_same(s1, domain_lists(big["x"], big["h"]))
    assert_same(s2, domain_lists(small["x"], small["h"]))
    assert np.array_equal(s1[0], s3[0]) and np.array_equal(s1[1], s3[1])


def test_static_search_rejects_sizes_beyond_its_scratch():
    torch = _torch()
    dev = torch.device("cuda:0")
    f = _entry()
    err = C.create_string_buffer(256)
    n = MAX_PARTICLES + 1
    xd = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    cd = torch.zeros(n, dtype=torch.int32, device=dev)
    ld = torch.zeros(n * NB, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert f(xd.data_ptr(), n, 1e-3, cd.data_ptr(), ld.data_ptr(), stream, err, 256) == -1
    assert b"65536" in err.value
    # two particles 10 m apart with h = 0.1 mm: the grid needs ~1e6 cells
    x2 = torch.tensor([0.0, 0.0, 0.0, 10.0, 0.0, 0.0], dtype=torch.float64, device=dev)
    assert f(x2.data_ptr(), 2, 1e-4, cd.data_ptr(), ld.data_ptr(), stream, err, 256) == -1
    assert b"262144" in err.value
    # host memory is refused before any device work
    xh = np.zeros(6)
    assert f(xh.ctypes.data, 2, 1e-3, cd.data_ptr(), ld.data_ptr(), stream, err, 256) == -1
    assert b"device-accessible" in err.value
    assert f(None, 0, 1e-3, None, None, stream, err, 256) == 0     # empty input
    # a rejected call leaves the entry point usable
    _, small = _cases()
    assert_same(static_lists(small["x"], small["h"]), domain_lists(small["x"], small["h"]))


def test_static_search_rejects_a_non_finite_position_in_any_block():
    """A NaN or Inf in the caller's positions (an ordinary input, it cannot fault
    the GPU) is rejected with WF_ERR_ARG on every call, wherever the particle
    sits: the status word that records it is cleared before the launch that
    checks the positions, not inside it."""
    torch = _torch()
    dev = torch.device("cuda:0")
    big, small = _cases()
    n = big["n"]
    assert n > 5000
    f = _entry()
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    cd = torch.zeros(n, dtype=torch.int32, device=dev)
    ld = torch.zeros(n * NB, dtype=torch.int32, device=dev)
    for k, (idx, bad) in enumerate([(5000, np.nan), (n - 1, np.inf), (5000, np.nan),
                                    (17, -np.inf), (12345, np.nan)]):
        x = np.array(big["x"], dtype=np.float64).reshape(-1, 3).copy()
        x[idx, k % 3] = bad
        xd = torch.from_numpy(x.reshape(-1)).to(dev)
        rc = f(xd.data_ptr(), n, big["h"], cd.data_ptr(), ld.data_ptr(), stream, err, 256)
        assert rc == -1, (idx, rc, err.value)
        assert b"not finite" in err.value
    # and a clean call right after gives the domain search's lists
    assert_same(static_lists(small["x"], small["h"]), domain_lists(small["x"], small["h"]))
