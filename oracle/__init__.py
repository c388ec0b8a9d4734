"""CPU ORACLE -- test infrastructure only; the product never imports this package.

A plain-C restatement of the reference (fractalyze/zorch) commit path:
Reed-Solomon coset LDE, Poseidon2 sponge/compression Merkle trees, the duplex
Fiat-Shamir transcript and FRI/Basefold fold rounds. Built by oracle/build.py.
"""
