/* empty: no configure step for the oracle build */
