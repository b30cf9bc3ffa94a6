// tdda_session.h -- cross-lattice FP32+refine solves with slot refill (library-internal).
//
// A "shape" holds the FFT work grid of one grid shape (Mx, My, Mz) for `cap`
// right-hand-side slots, but no lattice of its own: every slot brings a model
// whose own core (its lattice, Green spectrum and cellmap) shares that grid
// shape.  The FP32 inner solves of all slots run in one launch per pass (each
// right-hand side reads its own lattice through RhsVecs); each slot's FP64
// residual of the refinement runs on its own core.  Slots are admitted and
// released between rounds, so requests join a running batch as others finish
// (continuous batching).  Every slot's arithmetic is the same as its model's
// solve alone (tdda_model_solve_mixed), so its result is bit-identical to it.
//
// One thread drives a shape at a time.  Implemented in tdda_api.cu; used by
// tdda_solve_multi and the serving loop (tdda_server.cu).
#pragma once

#include <vector>

#include "../../include/tdda.h"

namespace tdda_session {

struct Shape;

struct Done {
    int slot;
    tdda_model* model;
    tdda_solve_info info;
};

// the FFT grid of a core; the device memory of a core of max_rhs right-hand
// sides, of one model, and of a shape of `cap` slots (upper estimates)
void core_grid(const tdda_core* c, int grid[3]);
int core_device(const tdda_core* c);
double core_bytes(int Nx, int Ny, int Nz, int N, int max_rhs);
double model_bytes(int N, int precision);
double shape_bytes(const int grid[3], int cap);
// the FFT grid a lattice box gets (tdda_core_create's choice)
void grid_of_box(int Nx, int Ny, int Nz, int grid[3]);

tdda_status shape_create(int device, const int grid[3], int cap, Shape** out);
void shape_destroy(Shape* s);
// whether a model's core can take a slot of the shape (same device and grid shape)
bool shape_accepts(const Shape* s, const tdda_model* m);
int shape_cap(const Shape* s);
int shape_active(const Shape* s);
// takes a free slot for model m (P as the model holds it: zero or a warm start);
// precond: its inner solves' preconditioning, 0 none, 1 Jacobi (TDDA_FP32_JACOBI),
// 2 chosen from the model's al (TDDA_FP32_AUTO)
tdda_status shape_admit(Shape* s, tdda_model* m, int max_it, double tol, int* slot, int precond = 0);
// One round: the refinement residual of every slot that needs one (on its own
// core), the start of the inner solves that follow, one launch of the
// device-side loop of the inner solves (at most 8 chunks of 4 steps), and the
// end of the inner solves that stopped.  Slots whose solve has ended are freed
// and appended to *done.
tdda_status shape_step(Shape* s, std::vector<Done>* done);

// A model's incident field and densities replaced in place (the buffers kept):
// the serving loop reuses the models of a cached operator.  P = 0.
tdda_status model_reinit(tdda_model* m, const double* nK, double E0, const double* nE0, const double* diel_old);

}  // namespace tdda_session
