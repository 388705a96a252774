"""Oracle package: TEST INFRASTRUCTURE, not the product.

CPU FP64 restatement of the reference hot path (fargo_oracle.cpp), its build
recipe (build.py), and the recipe that compiles the reference's own sources for
the CPU to pin it (ref_emul/).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may use it.
"""
