"""Simulation parameters and options with the reference drivers' defaults
(``initVes2D``, mytorch/driver_confined.py:14-77)."""
from __future__ import annotations

DEFAULT_PRAMS = {
    'N': 32, 'nv': 1, 'Nbd': 0, 'nvbd': 0, 'T': 1, 'dt': 1e-5, 'kappa': 1e-1, 'viscCont': 1,
    'gmresTol': 1e-5, 'gmresMaxIter': 1000, 'areaLenTol': 1e-2, 'repStrength': 900, 'minDist': 0.4,
    'farFieldSpeed': 1000, 'chanWidth': 2.5, 'vortexSize': 2.5,
}

DEFAULT_OPTIONS = {
    'farField': 'shear', 'repulsion': False, 'correctShape': False, 'reparameterization': False,
    'usePreco': True, 'matFreeWalls': False, 'confined': False,
}


def initVes2D(options=None, prams=None):
    """Fill missing ``options`` / ``prams`` entries with the defaults, zero the
    wall sizes of an unconfined run and expand a scalar ``viscCont`` to one
    entry per vesicle (mytorch/driver_confined.py:14-77).  The dicts are
    updated in place and returned, as in the reference."""
    options = {} if options is None else options
    prams = {} if prams is None else prams
    for key, val in DEFAULT_PRAMS.items():
        prams.setdefault(key, val)
    for key, val in DEFAULT_OPTIONS.items():
        options.setdefault(key, val)
    if not options['confined']:
        prams['Nbd'] = 0
        prams['nvbd'] = 0
    if isinstance(prams['viscCont'], (int, float)):
        prams['viscCont'] = [prams['viscCont']] * prams['nv']
    return options, prams
