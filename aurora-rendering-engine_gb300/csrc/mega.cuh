// mega.cuh — the megakernels' path loop over a 4-wide tree (render.cu:
// k_tail, guided_mega.cu: k_guided_tail), with the lanes' tree walks
// interleaved.
#pragma once

#include "path.cuh"

namespace are_core {

// lanes of a warp whose walks have ended hold their hits until this many of
// them (or every lane with a path, when no lane walks on) have one to shade
constexpr int WALK_READY_LANES = 20;

// Runs the queue entries i, i + stride, ... (< n) of this thread to the end
// over the 4-wide tree: each entry's path and, through `shade`, the paths its
// slot takes after it.  Every lane of the warp calls this (converged).
//
// The lanes' walks interleave.  Each round either the lanes at a wide node or
// the lanes at a leaf take one step (whichever are more; a tie goes to the
// leaves), so a round runs one kind of visit, and a lane whose walk has ended
// holds its hit until WALK_READY_LANES lanes have one; those shade together
// and begin their next walks.  Paths are traced and shaded exactly as
// closest_hit4 + shade would, so the image is the same bit for bit.
//
//   begin_entry(i): loads queue entry i into P (and whatever the caller keeps per entry)
//   shade(h):       one bounce of P at hit h = (t, leaf bits, u, v); true if P holds a ray to trace
//   end_entry():    the entry's slot has no sample left (write its sums back)
template <int SHORT, bool WIDE, class Begin, class Shade, class End>
__device__ __forceinline__ void interleaved_walks(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes,
	int4 *__restrict__ sstack, float tmin, unsigned i, unsigned n, unsigned stride, const PathState &P, uint32_t &err,
	unsigned long long &segments, Begin begin_entry, Shade shade, End end_entry) {
	const float inf = __int_as_float(0x7f800000);
	WalkStack<(WIDE ? MAX_STACK4 : MAX_STACK) - SHORT> st;
	Walk w;
	bool live = i < n, walking = false;
	if (live) {
		begin_entry(i);
		walking = WIDE ? walk4_begin(S, P.o, P.d, tmin, inf, w) : walk2_begin(S, snodes, n_snodes, P.o, P.d, tmin, inf, w);
	}
	while (__any_sync(0xffffffffu, live)) {
		for (;;) {
			const unsigned walkers = __ballot_sync(0xffffffffu, walking);
			const unsigned ready = __ballot_sync(0xffffffffu, live && !walking);
			if (walkers == 0 || __popc(ready) >= WALK_READY_LANES) break;
			const unsigned at_leaf = __ballot_sync(0xffffffffu, walking && w.b > 0);
			const bool leaf_round = 2 * __popc(at_leaf) >= __popc(walkers);
			if (walking && (w.b > 0) == leaf_round) {
				if constexpr (WIDE)
					walking = walk4_step<SHORT>(S, snodes, n_snodes, P.o, P.d, tmin, inf, err, sstack, st, w);
				else
					walking = walk2_step<SHORT>(S, snodes, n_snodes, P.o, P.d, tmin, inf, err, sstack, st, w);
			}
		}
		if (live && !walking) {
			++segments;
			live = shade(make_float4(w.best.t, __int_as_float(w.best.leaf), w.best.u, w.best.v));
			if (!live) {
				end_entry();
				i += stride;
				if (i < n) {
					begin_entry(i);
					live = true;
				}
			}
			if (live)
				walking = WIDE ? walk4_begin(S, P.o, P.d, tmin, inf, w) : walk2_begin(S, snodes, n_snodes, P.o, P.d, tmin, inf, w);
		}
	}
}

}  // namespace are_core
