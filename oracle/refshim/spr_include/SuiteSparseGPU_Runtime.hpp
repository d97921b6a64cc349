/* Stand-in (empty): sparse_relax.cpp includes it; nothing from it is used. */
