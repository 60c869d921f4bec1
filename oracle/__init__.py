"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the OSTR path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
package; the product path (newrecon_gb300) never does.
"""
