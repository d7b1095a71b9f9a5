"""cgs constants with the reference's literal values (mahakala/constants.py:22-31;
MP as in mahakala/electrons.py:25 and mahakala/grmhd/grmhd.py:28)."""

EE = 4.8032e-10
KB = 1.3807e-16
CL = 2.99792458e10
ME = 9.1094e-28
MP = 1.6726e-24
HPL = 6.6261e-27
GNEWT = 6.6743e-8

Msun = 1.989e33

# flux of an image: 1 Jy = 1e-23 erg s^-1 cm^-2 Hz^-1
JY = 1e-23
PARSEC = 3.0857e18
