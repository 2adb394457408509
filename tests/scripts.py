"""The reference's regression scripts, restated as functions of a simulation class.

Each function follows one script of pyranda/examples (the ones its test-suite
runs, tests/cases/*.py) and returns the scalar the script prints last.  The
simulation class is either the oracle's numpy restatement (``OracleSim``) or
the product's ``pyranda_gb300.pyrandaSim``; the scripts only use the API the
two share.  Mesh and EOM strings are the reference scripts' own inputs.
"""
import numpy

from pyranda_gb300.problems import TGV_EOM, TGV_IC, tgv_mesh  # noqa: F401  (problem strings)


def _f(x):
    """float() of a Python number, numpy scalar or 0-d torch tensor."""
    try:
        return float(x)
    except TypeError:
        return float(x.item())


def _sumsq_diff(a, b):
    d = a - b
    s = (d * d).sum()
    return _f(s)


def unit_test(Sim, **kw):
    """examples/unit_test.py: derivatives and filters on periodic and one-sided meshes."""
    ERROR = 0.0
    Nx = 32
    L = numpy.pi * 2.0 * (Nx - 1) / Nx
    domain = """
xdom = (0.0 , L , Nx ,periodic=True)
ydom = (0.0 , L , Nx ,periodic=True)
zdom = (0.0 , L , Nx ,periodic=True)
""".replace("L", str(L)).replace("Nx", str(Nx))
    pysim = Sim("advection", domain, **kw)
    expr = "sum( abs( ddx( sin(meshx) ) - cos(meshx) ))"
    for e in (expr, expr.replace("x", "y"), expr.replace("x", "z")):
        ERROR += _f(pysim.eval(e))
    domain = """
xdom = (0.0 , 1.0 , Nx )
ydom = (0.0 , 1.0 , Nx )
zdom = (0.0 , 1.0 , Nx )
""".replace("Nx", str(Nx))
    pysim2 = Sim("nonperiodic", domain, **kw)
    for expr in ("mean( abs(ddx(meshx*0.0)) )", "mean( abs(ddx(meshx*0.0 + 1.0)) )"):
        for e in (expr, expr.replace("x", "y"), expr.replace("x", "z")):
            ERROR += _f(pysim2.eval(e))
    expr = "mean( abs(ddx(meshx**power) - power*meshx**(power-1) )  )"
    for power in (1, 2, 3, 4):
        ex = expr.replace("power", str(float(power)))
        for e in (ex, ex.replace("x", "y"), ex.replace("x", "z")):
            ERROR += _f(pysim2.eval(e))
    groups = [
        (pysim2, ["mean( abs(fbar(meshx*0.0)) )", "mean( abs(fbar(meshx*0.0 + 1.0) - (meshx*0.0 + 1.0)  ) )",
                  "mean( abs(fbar(meshx) - (meshx)  ) )"]),
        (pysim, ["mean( abs(fbar(sin(meshx)) - sin(meshx)  ) )", "mean( abs(fbar( meshx*0.0 + 1.0) - 1.0  ) )",
                 "mean( abs(fbar( meshx*0.0 )  ) )"]),
        (pysim2, ["mean( abs(gbar(meshx*0.0)) )", "mean( abs(gbar(meshx*0.0 + 1.0) - (meshx*0.0 + 1.0)  ) )",
                  "mean( abs(gbar(meshx) - (meshx)  ) )"]),
        (pysim, ["mean( abs(gbar(sin(meshx)) - sin(meshx)  ) )", "mean( abs(gbar( meshx*0.0 + 1.0) - 1.0  ) )",
                 "mean( abs(gbar( meshx*0.0 )  ) )"]),
    ]
    for sim, exprs in groups:
        for e in exprs:
            ERROR += _f(sim.eval(e))
    return ERROR


def advection_1d(Sim, Npts, **kw):
    """examples/advection.py N 1: one period of periodic advection, sum of squared error."""
    L = numpy.pi * 2.0
    Lp = L * (Npts - 1.0) / Npts
    ss = Sim("advection", "xdom = (0.0, %s, %d, periodic=True)" % (repr(Lp), Npts), **kw)
    ss.EOM(" ddt(:phi:)  =  -:c: * ddx(:phi:) ")
    ss.setIC("""
r   = sqrt( (meshx-pi)**2  )
:phi: = 1.0 + 0.1 * exp( -(r/(pi/4.0))**2 )
:phi2: = 1.0*:phi:
:c:   = 1.0
""")
    v = 1.0
    dt_max = v / Npts * L * .90
    tt = L / v * 1.0
    dt = dt_max
    time = 0.0
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt_max, (tt - time))
    return _sumsq_diff(ss.variables["phi"].data, ss.variables["phi2"].data)


def make_tgv(Sim, Npts, timestep, **kw):
    from pyranda_gb300.problems import build_tgv
    return build_tgv(Sim, Npts, timestep, **kw)


def taylor_green(Sim, Npts, tstop, timestep, steps=None, **kw):
    """examples/TaylorGreen.py N 1: enstrophy ratio at t = tstop (CFL 0.5)."""
    ss = make_tgv(Sim, Npts, timestep, **kw)
    CFL = 0.5
    dt = ss.variables["dt"].data * CFL
    enst0 = ss.var("enst").sum()
    time = 0.0
    n = 0
    while (time < tstop) if steps is None else (n < steps):
        time = ss.rk4(time, dt)
        dt = ss.variables["dt"].data * CFL
        n += 1
    return _f(ss.var("enst").sum() / enst0)


EULER_1D = """
# Primary Equations of motion here
ddt(:rho:)  =  -ddx(:rho:*:u:)
ddt(:rhou:) =  -ddx(:rhou:*:u: + :p: - :tau:)
ddt(:Et:)   =  -ddx( (:Et: + :p: - :tau:)*:u: )
# Conservative filter of the EoM
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:Et:        =  fbar( :Et:   )
# Update the primatives and enforce the EOS
:u:         =  :rhou: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u:) ) * ( :gamma: - 1.0 )
# Artificial bulk viscosity (old school way)
:div:       =  ddx(:u:)
:beta:      =  gbar(abs(ring(:div:))) * :rho: * 7.0e-2
:tau:       =  :beta:*:div:
"""


def shu_osher_run(Sim, Npts, packages, **kw):
    """getShu of examples/shu_osher.py: returns (x, rho) at t = 1.8."""
    L = 10.0
    Lp = L * (Npts - 1.0) / Npts
    imesh = "xdom = (-Lp/2.0, Lp/2.0, Npts)".replace("Lp", str(Lp)).replace("Npts", str(Npts))
    ss = Sim("sod", imesh, **kw)
    packages(ss)
    eom = EULER_1D + """
# Apply constant BCs
bc.const(['u'],['xn'],0.0)
bc.const(['u'],['x1'],2.629369)
bc.const(['rho'],['x1'],3.857143)
bc.const(['p'],['x1'],10.33333)
bc.const(['Et'],['x1'],39.166585)
:rhou: = :rho:*:u:
:cs:  = sqrt( :p: / :rho: * :gamma: )
:dt: = dt.courant(:u:,0.0,0.0,:cs:)
:dt: = numpy.minimum(:dt:,0.2 * dt.diff(:beta:,:rho:))
"""
    ss.EOM(eom)
    ic = """
:gamma: = 1.4
eps = 2.0e-1
:tmp: = (meshx+4.0)/%s
:dum: = tanh(:tmp:)
:dum: = (:dum:+1.0)/2.0
:rho: = 3.857143 + :dum:*(1.0+eps*sin(5.0*meshx) - 3.857143)
:u: = 2.629369*(1.0-:dum:)
:p: = 10.33333 + :dum:*(1.0-10.33333)
:rhou: = :rho: * :u:
:Et:  = :p:/(:gamma: -1.0) + .5*:rho:*:u:*:u:
"""
    ss.setIC(ic % ss.dx)
    time = 0.0
    CFL = 0.5
    dt = _f(ss.variables["dt"].data) * CFL * .01
    tt = 1.8
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt * 1.1, _f(ss.variables["dt"].data) * CFL)
        dt = min(dt, (tt - time))
    x = _host(ss.variables["meshx"].data if "meshx" in ss.variables else ss.meshx)[:, 0, 0]
    rho = _host(ss.variables["rho"].data)[:, 0, 0]
    return x, rho


def _host(a):
    if hasattr(a, "cpu"):
        t = a.detach()
        return numpy.asfortranarray(t.permute(2, 1, 0).cpu().numpy().transpose(2, 1, 0))
    if hasattr(a, "data") and not isinstance(a, numpy.ndarray):
        return _host(a.data)
    return numpy.asarray(a)


def shu_osher(Sim, packages, **kw):
    """examples/shu_osher.py 1: average convergence rate of rho(1.85) over N = 100..800."""
    sol = []
    for n in (100, 200, 400, 800):
        x, rho = shu_osher_run(Sim, n, packages, **kw)
        sol.append(numpy.interp(1.85, x, rho))
    sol = numpy.array(sol)
    diff = numpy.abs(sol[1:] - sol[:-1])
    cr1 = numpy.log(diff[-1] / diff[-2]) / numpy.log(.5)
    cr2 = numpy.log(diff[-2] / diff[-3]) / numpy.log(.5)
    return float((cr1 + cr2) / 2.0)
