// flock/parameters.h -- compile-time defaults of the reference's switches
// (src/parameters.h, src/parallel_simplex_method/parallel_structs.h:34-89),
// mapped onto the runtime flock_options of the C ABI.
#pragma once
#include "../flock.h"

// BFS_METHOD: "vam_host" semantics (computed on the GPU), "nwc_host", or
// FLOCK_BFS_VOGEL_DEVICE for "vam_device" semantics.
#ifndef FLOCK_DEFAULT_BFS
#define FLOCK_DEFAULT_BFS FLOCK_BFS_VOGEL
#endif

// MAX_ITERATIONS: the reference caps simplex iterations at 30000.  Here the
// cap counts pricing rounds; 0 means no cap (the anti-cycling rule
// guarantees termination).
#ifndef MAX_ITERATIONS
#define MAX_ITERATIONS 0
#endif

// MAKE_WITH_GUROBI: the reference's build switch for its LP model
// (src/parameters.h); this library has no Gurobi model.
#ifndef MAKE_WITH_GUROBI
#define MAKE_WITH_GUROBI 0
#endif
