/* included by the reference but unused; empty stand-in */
