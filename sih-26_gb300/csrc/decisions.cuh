// decisions.cuh -- the scalar decisions of the restarted PDHG, shared by the FP64 loop and
// the FP32 inner loop of the mixed method. All of it runs on ONE device thread, in FP64.
#pragma once

#include "common.cuh"
#include "kernels.cuh"

namespace sgb {

// Called by every block of an evaluation's last kernel once it has read the flags: the last
// block to arrive clears them (and its ticket), after which the next step runs.
__device__ inline void clear_evaluation_flags(Ctl* c) {
  __shared__ bool s_last_apply;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last_apply = atomicAdd(&c->ticket[kTicketApply], 1u) == gridDim.x - 1;
    if (s_last_apply) {
      c->eval_now = 0;
      c->copy_best = 0;
      c->do_restart = 0;
      c->ticket[kTicketApply] = 0;
      __threadfence();
    }
  }
}

// The primal half of the movement for the row pass's decision (every thread of the last
// block calls it; thread 0 gets the value). When the column pass had no long column to
// finish, its blocks only published their partials and the sum is taken here, in block
// order as the column pass's own last block would have (`published` true); otherwise that
// block already left it in the control block. Either way ctl->mv_primal holds it after.
__device__ __forceinline__ double primal_movement(bool published, const double* part,
                                                  int nblocks, double omega, Ctl* ctl,
                                                  double* scratch) {
  if (!published) return ctl->mv_primal;
  double tp[1];
  sum_partials<1>(part, nblocks, scratch, tp);
  const double mv = 0.5 * omega * tp[0];
  if (threadIdx.x == 0) ctl->mv_primal = mv;
  return mv;
}

// Adaptive step, src/pdhg/pdhg.cpp:252-335: accept iff eta <= movement / interaction, then
// eta <- clamp(min(shrink * limit, grow * eta), 1e-12, ceiling) unless the step carried no
// information; an accepted step flips the current buffer and counts an iteration.
//
// The two factors depend only on the iteration count: shrink = 1 - e^-0.3 and grow = 1 + e^-0.6
// with e = max(iteration + 1, 2). step_factors() gives them; a kernel whose decision sits on
// its critical path (the last block's) reads them from a table filled once by the same pow
// (k_step_factors), so the decision does not wait on two FP64 pow calls on one thread.
__device__ inline long long step_factor_index(long long iteration) {
  return iteration + 1 > 2 ? iteration + 1 : 2;
}

__device__ inline double2 step_factors(long long e) {
  const double exponent = static_cast<double>(e);
  return make_double2(1.0 - pow(exponent, -0.3), 1.0 + pow(exponent, -0.6));
}

// The factors of iteration count `iteration` from `table` (n entries, indexed by e) where it
// covers e, else computed.
__device__ inline double2 step_factors(long long iteration, const double2* table, long long n) {
  const long long e = step_factor_index(iteration);
  return (table != nullptr && e < n) ? table[e] : step_factors(e);
}

__device__ inline void step_decision(Ctl* c, double movement, double interaction,
                                     double2 factors) {
  c->movement = movement;
  c->interaction = interaction;
  const bool no_information = interaction <= 0.0;
  const double limit = no_information ? __longlong_as_double(0x7ff0000000000000LL)
                                      : movement / interaction;
  const double shrink = factors.x;
  const double grow = factors.y;
  const double proposed = dmin(shrink * limit, grow * c->eta);
  const bool accept = c->eta <= limit;
  if (accept) {
    c->cur ^= 1;
    c->iteration += 1;
    c->averaged += 1;
    c->pending_add = 1;
  } else {
    c->pending_add = 0;
  }
  if (!no_information) {
    double eta = proposed;
    eta = eta < 1e-12 ? 1e-12 : (c->eta_ceiling < eta ? c->eta_ceiling : eta);
    c->eta = eta;
  }
  c->attempts += 1;
  c->accepted = accept;
  c->no_information = no_information;
  c->eval_now = (c->iteration > 0) && ((c->iteration % 40) == 0 || no_information);
}

__device__ inline void step_decision(Ctl* c, double movement, double interaction) {
  step_decision(c, movement, interaction, step_factors(step_factor_index(c->iteration)));
}

// The evaluation-tick decisions of src/pdhg/pdhg.cpp:349-483 given the assembled residuals
// of the current candidate and (if averaged > 0) of the average: the better one, the best
// so far, the stop test, the restart and the primal-weight update. `stop_here` is the
// caller's stopping test applied to the chosen candidate. dx2 / dy2 are the squared
// distances of the current iterate from the restart anchor. omega_lo / omega_hi clamp the
// primal weight (the reference uses 1e-6 and 1e6).
__device__ inline void tick_decisions(Ctl* c, const Residuals& cur, const Residuals* avg,
                                      bool (*stop_test)(const Ctl*, const Residuals&),
                                      double dx2, double dy2, double omega_lo,
                                      double omega_hi) {
  c->evaluations += 1;
  Residuals chosen = cur;
  int which = 1;
  if (avg != nullptr && worst(*avg) < worst(cur)) {
    chosen = *avg;
    which = 2;
  }
  int copy = 0;
  if (worst(chosen) < worst(c->best)) {
    c->best = chosen;
    copy = which;
  }
  {
    const long long slot = c->log_count % kLogRing;
    c->log[slot].iteration = c->iteration;
    c->log[slot].primal_objective = chosen.primal_objective;
    c->log[slot].primal = chosen.primal;
    c->log[slot].dual = chosen.dual;
    c->log[slot].gap = chosen.gap;
    c->log_count += 1;
  }
  if (stop_test(c, chosen)) {
    c->best = chosen;
    c->copy_best = which;
    c->done = kConverged;
    return;
  }
  c->copy_best = copy;
  if (c->use_restarts) {
    const double kkt = worst(chosen);
    const long long since = c->iteration - c->last_restart;
    const bool sufficient = kkt <= 0.2 * c->restart_kkt;
    const long long f36 = static_cast<long long>(0.36 * static_cast<double>(c->iteration));
    const bool artificial = since >= (f36 > 40 ? f36 : 40);
    if (sufficient || artificial) {
      const double dx_norm = sqrt(dx2);
      const double dy_norm = sqrt(dy2);
      if (dx_norm > 1e-12 && dy_norm > 1e-12) {
        const double theta = 0.5;
        double omega = exp(theta * log(dy_norm / dx_norm) + (1.0 - theta) * log(c->omega));
        omega = omega < omega_lo ? omega_lo : (omega_hi < omega ? omega_hi : omega);
        c->omega = omega;
      }
      c->do_restart = 1;
      c->averaged = 0;
      c->pending_add = 0;
      c->restart_kkt = kkt;
      c->last_restart = c->iteration;
      c->restarts += 1;
      if (c->inner_mode) c->done = kRestartRound;
    }
  }
}

}  // namespace sgb
