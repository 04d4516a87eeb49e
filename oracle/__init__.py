"""The oracle: a CPU (NumPy) restatement of apyib's CISD/MP2/SCF hot path.

Test infrastructure only.  Only tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py may import it, as the checker; the apyib_gb300
package never does.  Pinned against fixtures generated by the reference
itself (tests/golden/make_golden.py)."""
