"""Constants of the reference (geepee/config.py:11-16)."""
JITTER = 1e-5
GH_DEGREE = 10
PROP_MM = 'MM'
PROP_LIN = 'LIN'
PROP_MC = 'MC'
MC_NO_SAMPLES = 5
