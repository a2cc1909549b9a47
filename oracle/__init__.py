"""CPU oracle for the matching hot path - TEST INFRASTRUCTURE ONLY.

A C++ restatement of the reference's ppf::Detector::trainModel / matchScene (see
sm_oracle.cpp), wrapped with ctypes. Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it, always as the checker or the timed CPU baseline;
the product library never imports, links or calls it.
"""
from .pyoracle import (MatchParam, Oracle, OracleModel, TrainParam, build, lib,  # noqa: F401
                       MODE_GRID, MODE_REF)
