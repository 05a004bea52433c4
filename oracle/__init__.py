"""CPU oracle (test infrastructure only): restatement of the reference routines.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load this
package, and only as the checker or the timed CPU baseline -- never on the
product path."""
