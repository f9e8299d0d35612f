"""TEST INFRASTRUCTURE: CPU oracle for the MD hot path (see oracle/mdoracle.c and oracle/ref/).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may import this
package.  The product library never calls it."""
