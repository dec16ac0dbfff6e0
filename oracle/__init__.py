"""Test oracle for starflood_gb300 (TEST INFRASTRUCTURE ONLY, never the product)."""
