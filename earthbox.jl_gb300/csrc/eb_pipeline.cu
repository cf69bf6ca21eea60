// eb_pipeline.cu -- one marker cycle with the host copies overlapped with the steps.
//
// The cycle is MarkerInCell.marker_cycle's sequence of entry points (inside flags,
// bilinear set-up, heat scatter -- the weight denominators summed in the heat fold --,
// Stokes scatter, post-Stokes gathers, subgrid stress, stress correction, subgrid heat,
// remaining temperature change, RK4 advection, strain update), each of which the reference calls from its time loop
// (TimeLoop.jl; the call sites are listed beside each entry point in the header).
// Here the caller's host arrays go in and out inside the same call:
//   * uploads run on a copy stream in the order the steps first read them, in four
//     groups, each closed by an event; a step waits (on the device) only for the
//     group holding its inputs;
//   * downloads run on a second copy stream, each field as soon as the last step
//     that writes it has finished, so they overlap the remaining steps and the
//     uploads still in flight (the link is full duplex).
// The call returns after every copy and step has completed.
#include "eb_internal.h"

#include <algorithm>
#include <vector>

namespace {

// Steps of the cycle, in order.
// (the stress correction, remaining temperature change, advection and strain update run
// as one pass, eb_correct_advect_and_update_strain)
enum Step {
  ST_INSIDE = 0, ST_BILINEAR, ST_HEAT, ST_STOKES, ST_POST_STOKES, ST_SUBGRID_STRESS, ST_SUBGRID_HEAT, ST_TAIL,
  ST_COUNT
};

// Upload group of an input field: 0 positions and material (locate), 1 heat scatter,
// 2 Stokes scatter (and every later step but the strain update), 3 the rest.
int input_group(int f) {
  switch (f) {
    case EB_M_X: case EB_M_Y: case EB_M_MATID:
      return 0;
    case EB_M_TK: case EB_M_KT: case EB_M_RHOCP: case EB_M_HA: case EB_M_SERP_HR:
      return 1;
    case EB_M_RHO: case EB_M_COHESION: case EB_M_FRIC: case EB_M_ETA_FLOW: case EB_M_ETA: case EB_M_SXX:
    case EB_M_SXY: case EB_M_PFAILURE: case EB_M_DILATATION: case EB_M_MELTFRAC:
      return 2;
    default:
      return 3;
  }
}
// Inputs of group 3 that no step before the strain update reads.
bool read_only_by_strain(int f) { return f == EB_M_GII || f == EB_M_STRAIN_PLASTIC; }

// The last step writing an output field (after it the field is final).
int final_step(int f) {
  switch (f) {
    case EB_M_INSIDE: return ST_INSIDE;
    case EB_M_XN: case EB_M_YN: case EB_M_XN_VY: case EB_M_YN_VY: return ST_BILINEAR;
    case EB_M_EXX: case EB_M_EXY: case EB_M_PR: case EB_M_SR_RATIO: return ST_POST_STOKES;
    case EB_M_SUBGRID_DT: return ST_SUBGRID_HEAT;
    default: return ST_TAIL;  // tk, x, y, stresses, strains, velocities, and fields the cycle only reads
  }
}

int run_step(eb_ctx* c, int s) {
  switch (s) {
    case ST_INSIDE: return eb_get_marker_inside_flags(c);
    case ST_BILINEAR: return cycle_bilinear_setup(c);
    case ST_HEAT: return cycle_heat_and_denominators(c);
    case ST_STOKES: return eb_interpolate_marker_stokes_parameters_to_grid(c);
    case ST_POST_STOKES: return eb_post_stokes_marker_gathers(c);
    case ST_SUBGRID_STRESS: return eb_update_subgrid_stress(c);
    case ST_SUBGRID_HEAT: return eb_subgrid_heat_diffusion_update(c);
    default: return eb_correct_advect_and_update_strain(c);
  }
}

}  // namespace

extern "C" int eb_marker_cycle_host(eb_ctx* c, const eb_marker_io* io) {
  if (!c || !io) return EB_BAD_INPUT;
  if (io->n_in < 0 || io->n_out < 0 || (io->n_in > 0 && (!io->in_fields || !io->in_host)) ||
      (io->n_out > 0 && (!io->out_fields || !io->out_host)))
    return eb_fail(c, EB_BAD_INPUT, "eb_marker_io: counts and arrays do not match");
  for (int k = 0; k < io->n_in; ++k) {
    const int f = io->in_fields[k];
    if (f < 0 || f >= EB_M_NFIELDS || !io->in_host[k]) return eb_fail(c, EB_BAD_INPUT, "eb_marker_io: bad input field");
    if (f == EB_M_XN || f == EB_M_YN || f == EB_M_XN_VY || f == EB_M_YN_VY || f == EB_M_INSIDE)
      return eb_fail(c, EB_BAD_INPUT, "cell indices and inside flags are computed on the device (download only)");
  }
  for (int k = 0; k < io->n_out; ++k) {
    const int f = io->out_fields[k];
    if (f < 0 || f >= EB_M_NFIELDS || !io->out_host[k]) return eb_fail(c, EB_BAD_INPUT, "eb_marker_io: bad output field");
    if (f == EB_M_XN_VY || f == EB_M_YN_VY)
      return eb_fail(c, EB_BAD_INPUT, "eb_marker_cycle_host: download marker_xn_vy/yn_vy with eb_marker_download");
  }
  if (!c->have_grid || !c->have_params) return eb_fail(c, EB_NOT_READY, "grid and parameters must be set first");
  cudaSetDevice(c->device);
  int rc;
  for (int k = 0; k < io->n_in; ++k)
    if ((rc = ensure_marker_field(c, io->in_fields[k]))) return rc;
  for (int k = 0; k < io->n_out; ++k)
    if ((rc = ensure_marker_field(c, io->out_fields[k]))) return rc;
  if (!c->copy_in) EB_CK(c, cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking));
  if (!c->copy_out) EB_CK(c, cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking));
  while (c->pipe_events.size() < 4 + ST_COUNT) {
    cudaEvent_t e;
    EB_CK(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->pipe_events.push_back(e);
  }
  cudaEvent_t* group_done = c->pipe_events.data();       // [4]
  cudaEvent_t* step_done = c->pipe_events.data() + 4;    // [ST_COUNT]
  // nothing queued earlier on the compute stream may race with the uploads
  EB_CK(c, cudaStreamSynchronize(c->stream));

  // uploads, group by group
  bool matid_in = false, other_in = false;
  for (int g = 0; g < 4; ++g) {
    for (int k = 0; k < io->n_in; ++k) {
      const int f = io->in_fields[k];
      if (input_group(f) != g) continue;
      const size_t bytes = (size_t)c->M * (f == EB_M_MATID ? 2 : (f == EB_M_PFAILURE || f == EB_M_DILATATION ? 4 : 8));
      if (c->M > 0) EB_CK(c, cudaMemcpyAsync(c->mf[f], io->in_host[k], bytes, cudaMemcpyHostToDevice, c->copy_in));
      if (f == EB_M_MATID) matid_in = true;
      if (g == 3 && !read_only_by_strain(f)) other_in = true;
    }
    if (g == 0 && matid_in && c->M > 0) {
      c->matid_min = 0;
      c->matid_max = 0;
      if ((rc = launch_matid_range(c, c->copy_in))) return rc;
    }
    EB_CK(c, cudaEventRecord(group_done[g], c->copy_in));
  }
  if (matid_in && c->M > 0) {
    EB_CK(c, cudaEventSynchronize(group_done[0]));
    if ((rc = finish_matid_range(c))) {
      cudaStreamSynchronize(c->copy_in);
      return rc;
    }
  }

  // which outputs become final after which step
  std::vector<std::vector<int>> outs(ST_COUNT);
  for (int k = 0; k < io->n_out; ++k) outs[final_step(io->out_fields[k])].push_back(k);

  for (int s = 0; s < ST_COUNT; ++s) {
    int g = s <= ST_BILINEAR ? 0 : (s == ST_HEAT ? 1 : (s < ST_TAIL ? 2 : 3));
    if (g == 2 && other_in) g = 3;  // an input of unknown first reader: wait for everything
    EB_CK(c, cudaStreamWaitEvent(c->stream, group_done[g], 0));
    if ((rc = run_step(c, s))) {
      cudaStreamSynchronize(c->copy_in);
      cudaStreamSynchronize(c->copy_out);
      return rc;
    }
    if (!outs[s].empty() && c->M > 0) {
      EB_CK(c, cudaEventRecord(step_done[s], c->stream));
      EB_CK(c, cudaStreamWaitEvent(c->copy_out, step_done[s], 0));
      for (int k : outs[s]) {
        const int f = io->out_fields[k];
        const size_t bytes = (size_t)c->M * (f == EB_M_MATID ? 2 : (f == EB_M_INSIDE ? 1 :
                             (f == EB_M_PFAILURE || f == EB_M_DILATATION || f == EB_M_XN || f == EB_M_YN ? 4 : 8)));
        EB_CK(c, cudaMemcpyAsync(io->out_host[k], c->mf[f], bytes, cudaMemcpyDeviceToHost, c->copy_out));
      }
    }
  }
  EB_CK(c, cudaStreamSynchronize(c->copy_in));
  EB_CK(c, cudaStreamSynchronize(c->copy_out));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}
