/* empty: memory-debug header not used by the oracle build */
