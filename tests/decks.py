"""Input decks of the reference's own examples, restated as ParDeck objects.

Each function cites the Par.inp it restates (EXAMPLES/<name>/Par.inp of the
reference).  Used by the tests only.
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from sem2dpack_gb300.deck import (Fault, Material, ParDeck, Receivers,  # noqa: E402
                                  Sources, Time)


def lambs_problem():
    """EXAMPLES/LambsProblem/Par.inp:1-44.  The &TIME namelist ends at the
    first '/', so kind stays at its default 'leapfrog' (time.f90:138)."""
    return ParDeck(
        ngll=9, ndof=2, fmax=25.0, xlim=(0.0, 4.0e3), zlim=(-2.0e3, 0.0), nelem=(40, 20),
        materials=[Material(tag=1, rho=2000.0, cp=3200.0, cs=1847.5)],
        absorbing=[1, 2, 4],
        time=Time(kind="leapfrog", total_time=1.5, dt=0.5e-3, courant=0.5),
        sources=Sources(coords=[(1500.0, -50.0)], f0=10.0, onset=0.15, ampli=1.0, angle=0.0),
        receivers=Receivers(number=2, first=(2200.0, 0.0), last=(2700.0, 0.0), field="D"),
    )


def test_sh():
    """EXAMPLES/TestSH/Par.inp:1-33."""
    return ParDeck(
        ngll=6, ndof=1, fmax=1.25, xlim=(0.0, 30.0), zlim=(0.0, 30.0), nelem=(60, 60),
        materials=[Material(tag=1, rho=1.0, cp=1.7321, cs=1.0)],
        absorbing=[2, 3],
        time=Time(kind="leapfrog", total_time=35.0, courant=0.3),
        sources=Sources(coords=[(0.0, 0.0)], f0=0.5, onset=3.0, ampli=0.25, angle=0.0),
        receivers=Receivers(number=7, first=(0.0, 0.0), last=(30.0, 0.0), field="D", isamp=1),
    )


def anisotropic():
    """EXAMPLES/Anisotropic/Par.inp (Komatitsch, Barnes and Tromp 2000 fig. 7)."""
    return ParDeck(
        ngll=6, ndof=2, fmax=400.0e3, xlim=(-0.325, 0.325), zlim=(-0.325, 0.325),
        nelem=(130, 130),
        domains=[(1, (1, 65), (1, 130)), (2, (66, 130), (1, 130))],
        materials=[Material(tag=1, aniso=True, rho=7100.0, c11=16.5e10, c13=5.0e10,
                            c33=6.2e10, c55=3.96e10),
                   Material(tag=2, rho=7100.0, cp=4820.729884542206, cs=2361.665680982894)],
        absorbing=[],
        time=Time(kind="leapfrog", total_time=1.0e-4, dt=5.0e-8),
        sources=Sources(coords=[(-0.02, 0.0)], f0=170.0e3, onset=6.0e-6, ampli=1.0e13,
                        angle=180.0),
        receivers=Receivers(number=49, first=(-12.0e-2, -8.0e-2), last=(12.0e-2, -8.0e-2),
                            field="D", isamp=1),
    )


def inabox():
    """EXAMPLES/InaBox/Par.inp:1-60 (example 1, homogeneous box)."""
    return ParDeck(
        ngll=5, ndof=2, fmax=25.0, xlim=(-1.0e3, 1.0e3), zlim=(-1.0e3, 1.0e3), nelem=(40, 40),
        materials=[Material(tag=1, rho=2400.0, cp=3800.0, cs=2000.0)],
        absorbing=[1, 2, 3, 4],
        time=Time(kind="newmark", total_time=2.0, courant=0.3, beta=0.0, gamma=0.5),
        sources=Sources(coords=[(0.0, 0.0)], f0=5.0, onset=0.4, ampli=1.0, angle=0.0),
        receivers=Receivers(number=21, first=(-500.0, -1000.0), last=(-500.0, 1000.0), field="V"),
    )


def test_abso(zbottom, znel, stacey, ndof=2, total_time=1.5):
    """EXAMPLES/TestAbso/Par.inp.template:1-53 with the substitutions of
    EXAMPLES/TestAbso/run_test_PSV:1-9 (ZBOTTOM, ZNEL; NDOF=2, TT=1.5): a
    vertical Ricker force in a 6 x (2 - zbottom) km box absorbing on all
    four sides, 91 receivers on the line z = -1 km.  With zbottom = -1 km
    that line is the bottom boundary; with zbottom = -3 km it is inside, and
    the difference measures what the bottom boundary reflects."""
    return ParDeck(
        ngll=9, ndof=ndof, fmax=75.0, xlim=(-1.5e3, 4.5e3), zlim=(zbottom, 2.0e3), nelem=(120, znel),
        materials=[Material(tag=1, rho=2500.0, cp=5000.0, cs=2887.0)],
        absorbing=[1, 2, 3, 4], stacey=[1, 2, 3, 4] if stacey else [],
        time=Time(kind="leapfrog", total_time=total_time, courant=0.6),
        sources=Sources(coords=[(0.0, 0.0)], f0=30.0, onset=0.05, ampli=1.0e9, angle=90.0),
        receivers=Receivers(number=91, first=(0.0, -1.0e3), last=(4.5e3, -1.0e3), isamp=1, field="V"),
    )


def wave_box(ndof=2, phase="P", angle=0.0, stf=None, periodic=False, no_wave=(), tdelay=None):
    """A 2 x 1 km box (NGLL 5, 20 x 10 elements, homogeneous) with absorbing
    sides and an incident plane wave (&SRC_DEF mechanism='WAVE' + &SRC_WAVE
    angle, phase, src_wave.f90) with a 10 Hz Ricker; `periodic` makes the
    left and right sides periodic, so that a wave at normal incidence is
    one-dimensional."""
    from sem2dpack_gb300.deck import Stf  # noqa: F401
    dk = ParDeck(
        ngll=5, ndof=ndof, fmax=10.0, xlim=(0.0, 2000.0), zlim=(0.0, 1000.0), nelem=(20, 10),
        materials=[Material(tag=1, rho=2500.0, cp=5000.0, cs=2887.0)],
        absorbing=[1, 3] if periodic else [1, 2, 3, 4],
        time=Time(kind="leapfrog", total_time=0.5, courant=0.5),
        sources=Sources(coords=[(0.0, 0.0)], f0=10.0, onset=0.12, ampli=1.0, mechanism="WAVE",
                        wave_angle=angle, wave_phase=phase, stf=stf,
                        tdelay=None if tdelay is None else [tdelay]),
        receivers=Receivers(number=9, first=(200.0, 500.0), last=(1800.0, 500.0), field="V", isamp=1),
    )
    if periodic:
        dk.periodic = (2, 4)
    dk.no_wave = list(no_wave)
    return dk


def traction_box(ndof=2, hstf=None, vstf=None, h="N", v="N", tag=3):
    """A box with absorbing sides but one (&BC_DIRNEU with time-dependent
    tractions, bc_dirneu.f90:50-169) and no source."""
    absorbing = [t for t in (1, 2, 3, 4) if t != tag]
    dk = ParDeck(
        ngll=5, ndof=ndof, fmax=10.0, xlim=(0.0, 2000.0), zlim=(0.0, 1000.0), nelem=(20, 10),
        materials=[Material(tag=1, rho=2500.0, cp=5000.0, cs=2887.0)],
        absorbing=absorbing, dirneu=[(tag, h, v, True)],
        time=Time(kind="leapfrog", total_time=0.3, courant=0.5),
        receivers=Receivers(number=9, first=(200.0, 700.0), last=(1800.0, 300.0), field="V", isamp=1),
    )
    dk.dirneu_stf = {tag: (hstf, vstf)}
    return dk
