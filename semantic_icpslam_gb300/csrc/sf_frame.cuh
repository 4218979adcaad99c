// The frame loop's device control block and the per-frame bookkeeping of
// the device-driven forms: Tracker::Track's state machine after ComputeSE3
// and the frame's statistics.  They run in their own one-thread launches
// (k_sys_post, k_sys_stats in system.cu) where no frame kernel is at hand,
// and otherwise inside the frame's kernels: the persistent ICP kernel ends
// with sys_post (FramePost) and the frame's last raycast starts with
// sys_stats (FrameStatsArgs), which saves two launches per frame.
#ifndef SF_FRAME_CUH_
#define SF_FRAME_CUH_

#include "sf_kernels.cuh"

namespace sf {

struct SysDev {
  double last_pose[16];
  int state;       // state of the next frame: 1 initialise, 0 track, -1 lost (relocalise); ICP runs only in 0
  int run;         // this frame is tracked: mapping runs
  int accepted;
  int first;       // this frame was the initialisation frame
  int prev_state;  // state this frame ran in (Tracker::lastState once the frame is done)
  int missed;      // Tracker::noMissedFrames
  int relocalised; // this frame was relocalised
  int icp_ran;     // a ComputeSE3 ran this frame (its stats are reported)
  Cam cam;         // camera of this frame's mapping pass
};

// Tracker::Track's state machine (Tracking.cc:65-119) after one frame's
// attempt.  st: the state the frame ran in (1 initialise, 0 track, -1
// relocalise); prev: the state the previous frame ran in; ok: the
// attempt's result (ComputeSE3's acceptance in state 0, Relocalise's in
// state -1).  Returns whether the frame is tracked (SwapFrame, then the
// mapping stage), and sets the next frame's state and the missed-frame
// count: ten misses in a row make the tracker lost, and the first frame
// tracked after a relocalisation is not swapped (Track returns false).
SF_HD int track_transition(int st, int prev, int ok, int &next, int &missed) {
  if (st == 1) {
    next = 0;
    return 1;
  }
  if (st == 0) {
    next = 0;
    if (ok) {
      missed = 0;
      return prev != -1 ? 1 : 0;
    }
    if (++missed > 9) next = -1;
    return 0;
  }
  next = ok ? 0 : -1;
  return ok ? 1 : 0;
}

// Track() outcome (Tracking.cc:65-119) and the mapping camera
// (Frame::GpuRotation / GpuInvRotation / GpuTranslation, Frame.cc:626-645);
// when the frame is tracked, also the start of its allocation pass
// (alloc_frame_begin), which would otherwise be a launch of its own.
// A lost frame (state -1) relocalises only in the host-driven path of
// sf_system_grab with candidates registered; here it stays lost.
__device__ __forceinline__ void sys_post(SysDev *s, const TrackCtl &ctl, const Cam &tmpl, const FuseScratch &f) {
  const int st = s->state;
  const int ok = st == 0 ? ctl.accepted : 0;
  int next, missed = s->missed;
  const int tracked = track_transition(st, s->prev_state, ok, next, missed);
  s->first = st == 1 ? 1 : 0;
  s->accepted = st == 1 ? 1 : ok;
  if (st == 0 && tracked)
    for (int k = 0; k < 16; ++k) s->last_pose[k] = ctl.next_pose[k];
  s->prev_state = st;
  s->state = next;
  s->missed = missed;
  s->relocalised = 0;
  s->icp_ran = st == 0 ? 1 : 0;
  s->run = tracked;
  if (tracked) alloc_frame_begin(f);
  const double *P = s->last_pose;
  Cam c = tmpl;
  c.R.rx = mk3((float)P[0], (float)P[1], (float)P[2]);
  c.R.ry = mk3((float)P[4], (float)P[5], (float)P[6]);
  c.R.rz = mk3((float)P[8], (float)P[9], (float)P[10]);
  c.Rinv.rx = mk3((float)P[0], (float)P[4], (float)P[8]);
  c.Rinv.ry = mk3((float)P[1], (float)P[5], (float)P[9]);
  c.Rinv.rz = mk3((float)P[2], (float)P[6], (float)P[10]);
  c.t = mk3((float)P[3], (float)P[7], (float)P[11]);
  s->cam = c;
}

// `host_out` (pinned host memory, or null) receives a copy, and then
// *host_ready the frame's sequence number, *seq + 1, which *seq keeps
// (stores from the kernel cost the frame less than a copy node and an
// event).  A reader waits for its own frame's number, so a flag left by an
// earlier frame that nobody waited for cannot stand in for it.
__device__ __forceinline__ void sys_stats(const SysDev *s, const TrackCtl &ctl, const DevMap &m,
                                          const uint32_t *flags, sf_frame_stats *out, sf_frame_stats *host_out,
                                          uint32_t *host_ready, uint32_t *seq) {
  sf_frame_stats st;
  st.tracked = s->run;
  st.accepted = s->accepted;
  st.state = s->state;
  st.missed = s->missed;
  st.relocalised = s->relocalised;
  if (!s->icp_ran) {  // no ComputeSE3 ran this frame
    st.fail = 0; st.iterations = 0; st.icp_error = 0.f; st.icp_count = 0;
    st.rgb_error = 0.f; st.rgb_count = 0;
  } else {
    st.fail = ctl.timeout ? 3 : ctl.stop;
    st.iterations = ctl.iters_run;
    st.icp_error = ctl.icpError;
    st.icp_count = ctl.icpCount;
    st.rgb_error = ctl.rgbError;
    st.rgb_count = ctl.rgbCount;
  }
  st.visible = s->run ? *m.no_visible : 0u;
  st.heap_counter = *m.heap_counter;
  st.entry_ptr = *m.entry_ptr;
  st.allocated = *m.alloc_count;
  st.flags = *flags;
  for (int k = 0; k < 16; ++k) st.pose[k] = s->last_pose[k];
  *out = st;
  if (host_out) {
    const uint32_t q = *seq + 1u;
    *seq = q;
    *host_out = st;
    __threadfence_system();  // the stats before the flag, as the host sees them
    *(volatile uint32_t *)host_ready = q;
  }
}

// sys_post's arguments for a kernel that runs it (sys null: it does not).
struct FramePost {
  SysDev *sys;
  Cam tmpl;
  FuseScratch f;
};

// sys_stats's arguments for a kernel that runs it (sys null: it does not).
struct FrameStatsArgs {
  const SysDev *sys;
  const TrackCtl *ctl;
  const uint32_t *flags;
  sf_frame_stats *out;
  sf_frame_stats *host_out;
  uint32_t *host_ready;
  uint32_t *seq;
};

}  // namespace sf
#endif
