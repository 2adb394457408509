"""Host logic of the EOM/IC string language (pyranda/pyrandaUtils.py:22-141)."""
from pyranda_gb300.pyrandaUtils import findVar, fortran3d, splitLines


def test_find_scalars_and_vectors():
    line = "ddt(:rhou:) = -ddx(:rhou:*:u: - :tauxx:) + :[vel]:"
    assert sorted(findVar(line, "scalar")) == ["rhou", "tauxx", "u"]
    assert findVar(line, "vector") == ["vel"]
    assert findVar("[:tx:,:ty:,:tz:] = grad(:T:)", "scalar", unique=False) == ["tx", "ty", "tz", "T"]


def test_translation_order_and_variables():
    smap = {"ddx(": "self.ddx(", "abs(": "numpy.abs(", "sqrt(": "numpy.sqrt(", "pi": "numpy.pi"}
    out = fortran3d(":p: = sqrt( abs(:Et:) ) * pi + ddx(:u:)", smap)
    assert out == 'self.variables["p"].data=numpy.sqrt(numpy.abs(self.variables["Et"].data))*numpy.pi+self.ddx(self.variables["u"].data)'
    # the variable entries are appended to the map, as the reference does
    assert ':u:' in smap and list(smap)[-1].startswith(":")


def test_split_lines_drops_comments_and_blanks():
    assert splitLines("\n# comment\n:a: = 1\n\n  :b: = 2 \n") == [":a:=1", ":b:=2"]


def test_sim_smap_matches_reference_keys():
    """Every key of pyranda.py:812-869 is present, in the same order."""
    import pyranda_gb300.pyranda as P
    keys = list(P.pyrandaSim.get_sMap.__code__.co_consts)
    ref = ["div(", "ddx(", "ddy(", "ddz(", "fbar(", "gbar(", "gbarx(", "gbary(", "gbarz(", "grad(", "simtime",
           "deltat", "ring(", "ringV(", "dd8x(", "dd8y(", "dd8z(", "sum(", "mean(", "mean3D(", "sign(", "dot(",
           "abs(", "sqrt(", "sin(", "cos(", "tanh(", "exp(", "where(", "max(", "min(", "3d(", "pi", "gridLen",
           "random3D()", "erf(", "meshx", "meshy", "meshz", "meshi", "meshj", "meshk"]
    found = [k for k in keys if isinstance(k, str) and k in ref]
    assert found == ref


def test_kh_sizes_are_seeded():
    """The ensemble's member sizes: 64 draws from {128,...,512} by default_rng(seed=0)."""
    from pyranda_gb300.problems import kh_sizes
    s = kh_sizes()
    assert len(s) == 64 and set(s) <= {128, 192, 256, 384, 512}
    assert s == kh_sizes()
