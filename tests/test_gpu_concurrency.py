"""Concurrent calls: two host threads, each on its own CUDA stream, sharing
one octree and one cosmology handle (read-only after creation).  The
persistent fast kernel keeps one work-queue counter per (device, stream), so
the two launches may overlap; each thread's results equal those of the same
batch traced alone."""
import ctypes as C
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_two_streams_share_the_handles(gpu_lib, pkg, golden):
    torch = pytest.importorskip("torch")
    from importlib import import_module
    capi = import_module(pkg.__name__ + ".capi")
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    length = float(golden["cosmo_length"])
    base = np.asarray(golden["launch"], dtype=np.float64)
    # two different batches: the golden rays and the same rays mirrored in y
    batches = [np.tile(base, (16, 1)), np.tile(base * np.array([1, -1, 1, 1, -1, 1.0]), (16, 1))]
    ref = [pkg.propagate(tree, cos, b, length, nsteps=int(golden["nsteps"]), order=2, stop="redshift",
                         stop_value=float(golden["zs"][-1]), exact=False, jacobian=True)[0] for b in batches]
    p, keep = capi.make_params(length, int(golden["nsteps"]), 2, "redshift", float(golden["zs"][-1]), None, True, False, 0)
    L = pkg.library()
    dev = torch.device("cuda", 0)
    out = [None, None]
    errors = []

    def lane(j):
        try:
            torch.cuda.set_device(0)
            s = torch.cuda.Stream(dev)
            n = batches[j].shape[0]
            d_l = torch.from_numpy(batches[j]).to(dev)
            d_s = torch.zeros(n, dtype=torch.int64, device=dev)
            d_st = torch.zeros(1, dtype=torch.int32, device=dev)
            torch.cuda.synchronize()
            for _ in range(3):
                rc = L.mpf_propagate_device(tree._h, cos._h, C.byref(p), n, C.c_void_p(d_l.data_ptr()),
                                            C.c_void_p(d_s.data_ptr()), None, None, C.c_void_p(d_st.data_ptr()),
                                            C.c_void_p(s.cuda_stream))
                if rc < 0:
                    raise RuntimeError(rc)
            s.synchronize()
            out[j] = d_s.cpu().numpy()
        except Exception as e:   # reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=lane, args=(j,)) for j in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for j in range(2):
        np.testing.assert_array_equal(out[j], ref[j])
    del keep
    tree.close()
    cos.close()


def test_propagate_captured_in_a_cuda_graph(gpu_lib, pkg, golden):
    """mpf_propagate_device on a stream is capturable in a CUDA graph once the
    stream has seen one call (its work-queue counter and, for a batch of at
    least 2^17 rays, the autotuned shape exist then): the graph's replays
    (queue reset + the persistent launch) give the direct call's results,
    also after the launch records change in place."""
    torch = pytest.importorskip("torch")
    from importlib import import_module
    capi = import_module(pkg.__name__ + ".capi")
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    length = float(golden["cosmo_length"])
    base = np.asarray(golden["launch"], dtype=np.float64)
    zs = np.asarray(golden["zs"], dtype=np.float64)
    batches = [np.tile(base, (600, 1)), np.tile(base * np.array([1, -1, 1, 1, -1, 1.0]), (600, 1))]
    n = batches[0].shape[0]
    assert n >= (1 << 17)
    kw = dict(nsteps=int(golden["nsteps"]), order=2, stop="redshift", planes=zs, jacobian=True, exact=False)
    ref = [pkg.propagate(tree, cos, b, length, **kw) for b in batches]
    p, keep = capi.make_params(length, int(golden["nsteps"]), 2, "redshift", 0.0, zs, True, False, 0)
    L = pkg.library()
    dev = torch.device("cuda", 0)
    s = torch.cuda.Stream(dev)
    d_l = torch.from_numpy(batches[0]).to(dev)
    d_s = torch.zeros(n, dtype=torch.int64, device=dev)
    d_p = torch.zeros(n * zs.shape[0] * capi.MPF_PLANE_FIELDS, dtype=torch.float64, device=dev)
    d_st = torch.zeros(1, dtype=torch.int32, device=dev)

    def call():
        capi.check(L.mpf_propagate_device(tree._h, cos._h, C.byref(p), n, C.c_void_p(d_l.data_ptr()),
                                          C.c_void_p(d_s.data_ptr()), None, C.c_void_p(d_p.data_ptr()),
                                          C.c_void_p(d_st.data_ptr()), C.c_void_p(s.cuda_stream)))

    with torch.cuda.stream(s):
        call()                      # first call on the stream: queue counter and tuned shape
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        call()
    for j in (0, 1, 0):
        d_l.copy_(torch.from_numpy(batches[j]))
        d_s.zero_()
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_s.cpu().numpy(), ref[j][0])
        got = d_p.cpu().numpy().reshape(n, zs.shape[0], capi.MPF_PLANE_FIELDS)
        np.testing.assert_array_equal(got.view(np.uint64), ref[j][2].view(np.uint64))
    tree.close()
    cos.close()


def test_host_buffer_calls_from_two_threads(gpu_lib, pkg, golden):
    """mpf_propagate from two host threads at once (each thread gets its own
    stream inside the library): each thread's results equal the same batch
    traced alone."""
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    length = float(golden["cosmo_length"])
    base = np.asarray(golden["launch"], dtype=np.float64)
    batches = [np.tile(base, (64, 1)), np.tile(base * np.array([1, -1, 1, 1, -1, 1.0]), (64, 1))]
    kw = dict(nsteps=int(golden["nsteps"]), order=2, stop="redshift", stop_value=float(golden["zs"][-1]),
              exact=False, jacobian=True)
    ref = [pkg.propagate(tree, cos, b, length, **kw) for b in batches]
    out, errors = [None, None], []

    def lane(j):
        try:
            for _ in range(3):
                out[j] = pkg.propagate(tree, cos, batches[j], length, **kw)
        except Exception as exc:   # reported below
            errors.append(exc)

    th = [threading.Thread(target=lane, args=(j,)) for j in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for j in range(2):
        np.testing.assert_array_equal(out[j][0], ref[j][0])
        np.testing.assert_array_equal(out[j][1].view(np.uint64), ref[j][1].view(np.uint64))
    tree.close()
    cos.close()
