"""libgpx C ABI without a GPU: it loads, exports every declared symbol, parses
models and reports errors as status codes (no compute calls)."""
import os
import re
import subprocess

import pytest

from gpuexplore_gb300 import gen, gpf

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gpx.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(gpx_[a-z_]+)\s*\(", text)))


def test_exports_every_declared_symbol(built):
    import ctypes
    lib = ctypes.CDLL(built.LIB)
    missing = [s for s in _declared() if not hasattr(lib, s)]
    assert not missing, missing
    assert len(_declared()) >= 15


def test_model_info_matches_header(built, tmp_path):
    from gpuexplore_gb300 import lib
    for net in (gen.ring(1), gen.random_network(2), gen.random_network(3, nprocs=24, states=(4, 9))):
        p = tmp_path / "m.gpf"
        gpf.write(net, str(p))
        m = lib.Model.from_file(str(p))
        inf = m.info()
        h = gpf.header(gpf.encode(net))
        assert inf.nr_procs == h.nr_procs and inf.bits_act == h.bits_act
        assert inf.bits_statevector == h.bits_statevector and inf.nr_trans == h.nr_trans
        assert list(inf.firstbit[:h.nr_procs + 1]) == h.firstbit
        assert inf.state_bits == h.firstbit[-1]
        assert inf.key_words == (h.firstbit[-1] + 31) // 32
        m2 = lib.Model.from_words(gpf.encode(net))
        assert m2.info().nr_trans == inf.nr_trans


def test_parse_errors(built, tmp_path):
    from gpuexplore_gb300 import lib
    with pytest.raises(lib.GpxError) as e:
        lib.Model.from_file(str(tmp_path / "nope.gpf"))
    assert e.value.status == 1
    with pytest.raises(lib.GpxError) as e:
        lib.Model.from_words([0, 2, 3])
    assert e.value.status == 1
    words = gpf.encode(gen.ring(1))
    with pytest.raises(lib.GpxError):
        lib.Model.from_words(words[:-3])  # truncated rules
    wide = gen.random_network(1, nprocs=30, states=(17, 30), safety=False)  # 150 state bits
    with pytest.raises(lib.GpxError) as e:
        lib.Model.from_words(gpf.encode(wide))
    assert e.value.status == 7  # GPX_ERR_UNSUPPORTED


def test_status_strings(built):
    from gpuexplore_gb300 import lib
    L = lib.load()
    assert L.gpx_status_string(4) == b"problem with hash table"
    assert L.gpx_abi_version() == lib.ABI_VERSION == 4


def test_no_gpu_is_a_status(built, tmp_path):
    from gpuexplore_gb300 import lib
    if lib.device_info(0) is not None:
        pytest.skip("a GPU is present")
    p = tmp_path / "m.gpf"
    gpf.write(gen.ring(1), str(p))
    r = lib.explore(str(p), check=False)
    assert r["rc"] == 2


def test_cli_surface(built, tmp_path):
    cli = built.CLI
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "No input network given" in r.stderr
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage: gpuexplore" in r.stdout
    for flag in ("--por", "--cycle-proviso", "--ample", "--stubborn", "--por-model", "--dump", "-k", "-q",
                 "--no-prune"):
        assert flag in r.stdout, flag
    r = subprocess.run([cli, str(tmp_path / "x"), "-z"], capture_output=True, text=True)
    assert r.returncode == 1 and "unrecognized option -z" in r.stderr
    r = subprocess.run([cli, str(tmp_path / "x")], capture_output=True, text=True)
    assert r.returncode == 1 and "input network does not exist" in r.stderr
    gpf.write(gen.ring(1), str(tmp_path / "ring.gpf"))
    r = subprocess.run([cli, str(tmp_path / "ring"), "-p"], capture_output=True, text=True)
    assert "Property to check is not a liveness property" in r.stdout
    assert "nr of procs: 8" in r.stdout and "statevector offset 8: 24" in r.stdout


def test_option_validation_before_device(built, tmp_path):
    """Malformed options are refused before any device is touched (works without a GPU)."""
    from gpuexplore_gb300 import lib
    p = tmp_path / "m.gpf"
    gpf.write(gen.ring(1), str(p))
    bads = (dict(por=5), dict(por=-1), dict(bucket_bytes=64), dict(property=7), dict(threads=48),
            dict(threads=512), dict(q_words=1 << 62), dict(store_states=1 << 62))
    for bad in bads:
        r = lib.explore(str(p), check=False, **bad)
        assert r["rc"] == 6, bad  # GPX_ERR_INVALID
    # the allocation-free entry point refuses the same options the same way
    m = lib.Model.from_file(str(p))
    try:
        for bad in bads:
            r = lib.explore_noalloc(m, check=False, **bad)
            assert r["rc"] == 6, bad
    finally:
        m.close()


def test_option_defaults(built):
    from gpuexplore_gb300 import lib
    L = lib.load()
    o = lib.Options()
    L.gpx_options_init(lib.C.byref(o))
    assert o.launch_graph == 1 and o.por == 0 and o.kernel_iters == 0 and o.bucket_bytes == 0
    assert o.prune_commuting == 1 and o.set_hash == 0 and o.struct_size == lib.C.sizeof(lib.Options)
    b = lib.BatchOptions()
    L.gpx_batch_options_init(lib.C.byref(b))
    assert b.latency_sms == -1 and b.struct_size == lib.C.sizeof(lib.BatchOptions)
    assert b.prune_commuting == 1


def test_batch_option_validation(built, tmp_path):
    """gpx_batch_explore refuses bad launch options before it looks for a GPU."""
    from gpuexplore_gb300 import lib
    p = tmp_path / "m.gpf"
    gpf.write(gen.ring(1), str(p))
    m = lib.Model.from_file(str(p))
    try:
        for bad in (dict(threads=48), dict(threads=512), dict(threads=-32), dict(load_factor=0.99)):
            items, stats = lib.batch_explore([m], [{"property": "deadlock"}], check=False, **bad)
            assert stats["rc"] == 6, bad  # GPX_ERR_INVALID
    finally:
        m.close()


def test_wide_local_state_fields_decode_in_bounded_memory(built):
    """A process whose declared bits_state far exceeds its state count: the
    decoder's reachability array is bounded by the gpf's offset fields, not by
    2^bits_state (which would be 2^27 entries here)."""
    import time
    from gpuexplore_gb300 import lib
    net = gen.ring(1, nprocs=3, nstates=3)
    net.bits_state = lambda: [27, 2, 2]
    words = gpf.encode(net)
    t0 = time.perf_counter()
    m = lib.Model.from_words(words)
    elapsed = time.perf_counter() - t0
    try:
        assert m.info().state_bits == 31
    finally:
        m.close()
    assert elapsed < 0.1
