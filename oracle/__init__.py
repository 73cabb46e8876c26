"""CPU oracle of the implicit cloth step: test infrastructure only (the checker).

oracle/cloth_oracle.c  - FP64 restatement of the reference step (libcloth_oracle.so)
oracle/oracle.py       - its ctypes front
oracle/Makefile        - builds the reference's own CPU cloth code into oracle/_ref/
oracle/ref_harness.cpp - drives that build to produce the golden fixtures
"""
