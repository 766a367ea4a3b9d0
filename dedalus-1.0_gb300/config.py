"""Configuration keys of the reference (dedalus/config.py:29-56) that the hot
path reads, with the CUDA backend as the default FFT method.

Keys: ``FFT.method`` ('cuda'), ``FFT.dealiasing`` ('2/3 cython', '2/3',
'None'), ``FFT.precision`` ('fp64' | 'df64' | 'fp32': transform and nonlinear-product
arithmetic; df64 = double-float on the FP32 pipes, 3D hydro only), ``physics.use_tracer``, ``physics.boussinesq_direction``.  User
files ``~/.dedalus/config`` and ``./dedalus.cfg`` override the defaults, as in
the reference.
"""
import configparser
import os

decfg = configparser.ConfigParser()
decfg.add_section('FFT')
decfg.set('FFT', 'method', 'cuda')
decfg.set('FFT', 'dealiasing', '2/3 cython')
decfg.set('FFT', 'precision', 'fp64')
decfg.add_section('physics')
decfg.set('physics', 'use_tracer', 'False')
decfg.set('physics', 'boussinesq_direction', 'z')
decfg.read([os.path.expanduser('~/.dedalus/config'), 'dedalus.cfg'])


def precision_code():
    p = decfg.get('FFT', 'precision').lower()
    if p == 'fp64':
        return 0
    if p == 'fp32':
        return 1
    if p == 'df64':
        return 2
    raise NotImplementedError("FFT.precision must be fp64, df64 or fp32 (got %r)" % p)
