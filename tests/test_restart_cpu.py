"""Restart files in pyranda's format (pyranda/pyranda.py:475-589, 979-1130), on the CPU.

The writer's proc-00000.bin must be byte for byte what the reference's
writer produces for the same variables (an F-ordered (ax, ay, az, nvars)
array written with ndarray.tofile), serial.dat must evaluate to the same
dict, and the reader must assemble restarts of several blocks placed by
procMap, as the reference's readChunk does.
"""
import os

import numpy

from pyranda_gb300 import restart


def _vars(shape, seed=0):
    r = numpy.random.default_rng(seed)
    return {"rho": numpy.asfortranarray(r.random(shape)), "u": numpy.asfortranarray(r.standard_normal(shape)),
            "gamma": 1.4}


def test_block_bytes_match_the_reference_layout(tmp_path):
    shape = (6, 5, 4)
    v = _vars(shape)
    serial = {"mesh": {"nn": list(shape)}, "EOM": "", "ICs": "", "decomp": [1, 1, 1],
              "procMap": {"0-g1": numpy.zeros(3, dtype=numpy.int32),
                          "0-gn": numpy.array([5, 4, 3], dtype=numpy.int32)},
              "packages": [], "time": 0.5, "deltat": 0.1, "cycle": 7, "vizDumpHistory": [], "sMap": {"a": "b"}}
    d = str(tmp_path / "restart_0000007")
    restart.write_files(d, serial, v, shape)
    # the reference's writer: emptyVector(n) then DATA[:,:,:,slot] = data; DATA.tofile
    names = sorted(v)
    ref = numpy.zeros(shape + (len(names),), dtype=numpy.float64, order="F")
    for i, n in enumerate(names):
        ref[:, :, :, i] = v[n]
    ref_path = str(tmp_path / "ref.bin")
    with open(ref_path, "wb") as f:
        ref.tofile(f)
    assert open(os.path.join(d, "proc-00000.bin"), "rb").read() == open(ref_path, "rb").read()
    s = restart.read_serial(d)
    assert s["vars"] == {n: i for i, n in enumerate(names)} and s["cycle"] == 7 and s["sMap"] == {"a": "b"}
    assert numpy.array_equal(s["procMap"]["0-gn"], [5, 4, 3])
    back = restart.read_blocks(d, s, shape)
    assert numpy.array_equal(back["rho"], v["rho"]) and numpy.array_equal(back["u"], v["u"])
    assert numpy.all(back["gamma"] == 1.4)


def test_reader_assembles_blocks_of_a_decomposed_run(tmp_path):
    """Two ranks split x in halves, each block written the reference's way."""
    shape = (8, 3, 2)
    v = _vars(shape, 1)
    names = sorted(v)
    d = tmp_path / "restart_0000001"
    d.mkdir()
    procmap = {}
    for rank, (i0, i1) in enumerate(((0, 4), (4, 8))):
        blk = numpy.zeros((4, 3, 2, len(names)), order="F")
        for k, n in enumerate(names):
            blk[:, :, :, k] = (v[n][i0:i1] if isinstance(v[n], numpy.ndarray) else v[n])
        with open(d / ("proc-%s.bin" % str(rank).zfill(5)), "wb") as f:
            blk.tofile(f)
        procmap["%d-g1" % rank] = numpy.array([i0, 0, 0], dtype=numpy.int32)
        procmap["%d-gn" % rank] = numpy.array([i1 - 1, 2, 1], dtype=numpy.int32)
    serial = {"decomp": [2, 1, 1], "procMap": procmap, "vars": {n: i for i, n in enumerate(names)}}
    with open(d / "serial.dat", "w") as f:
        numpy.set_printoptions(threshold=10 ** 9)
        f.write(str(serial))
    s = restart.read_serial(str(d))
    back = restart.read_blocks(str(d), s, shape)
    assert numpy.array_equal(back["rho"], v["rho"]) and numpy.array_equal(back["u"], v["u"])
    assert restart.find_dump(str(tmp_path)) == str(d)
