// Host-side planner for split/consolidate job lists (no CUDA).
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace mamr {

// Runs a list of data-movement jobs with the reference's sequential
// semantics in as few launches as possible.  The reference places a later
// child (split) or target (consolidate) in the lowest free slot, which is
// usually one an earlier job of the same call just read and freed: a
// write-after-read hazard.  Jobs are cut into segments; inside a segment no
// job reads or writes a slot an earlier job of the segment wrote, and every
// slot a job of the segment overwrites after it was read is copied to a
// staging area before the segment runs, its readers redirected there
// (negative slot).  One segment is one staging copy plus one launch; the
// split and consolidation lists miniAMR produces fit one segment unless the
// staging budget runs out.
struct Segment {
   size_t begin, end;            // jobs [begin, end)
   size_t stage_begin, stage_end; // staged slots [stage_begin, stage_end)
};

template <int NR, int NW, typename Job, typename Reads, typename Writes>
static void plan_segments(std::vector<Job> &jobs, int max_slots,
                          size_t max_stage, Reads reads, Writes writes,
                          std::vector<int32_t> &staged,
                          std::vector<Segment> &segs)
{
   std::vector<int> seg_r(max_slots, -1), seg_w(max_slots, -1),
      seg_s(max_slots, -1);
   std::vector<int32_t> stage_idx(max_slots, 0);
   staged.clear();
   segs.clear();
   int cur = 0;
   Segment sg{0, 0, 0, 0};
   auto close = [&](size_t end) {
      sg.end = end;
      sg.stage_end = staged.size();
      for (size_t t = sg.begin; t < sg.end; t++)
         for (int32_t *r : reads(jobs[t]))
            if (*r >= 0 && seg_s[*r] == cur)
               *r = -1 - (stage_idx[*r] - (int32_t) sg.stage_begin);
      segs.push_back(sg);
      cur++;
      sg = Segment{end, end, staged.size(), staged.size()};
   };
   for (size_t t = 0; t < jobs.size(); t++) {
      std::array<int32_t *, NR> rd = reads(jobs[t]);
      std::array<int32_t *, NW> wr = writes(jobs[t]);
      auto own_read = [&](int32_t s) {
         for (int32_t *r : rd)
            if (*r == s)
               return true;
         return false;
      };
      bool conflict = false;
      for (int32_t *r : rd)
         conflict |= seg_w[*r] == cur;
      size_t need = 0;
      for (int32_t *w : wr) {
         conflict |= seg_w[*w] == cur;
         need += (seg_r[*w] == cur || own_read(*w)) && seg_s[*w] != cur;
      }
      if (t > sg.begin &&
          (conflict || staged.size() - sg.stage_begin + need > max_stage))
         close(t);
      for (int32_t *w : wr)
         if ((seg_r[*w] == cur || own_read(*w)) && seg_s[*w] != cur) {
            seg_s[*w] = cur;
            stage_idx[*w] = (int32_t) staged.size();
            staged.push_back(*w);
         }
      for (int32_t *r : rd)
         seg_r[*r] = cur;
      for (int32_t *w : wr)
         seg_w[*w] = cur;
   }
   if (!jobs.empty())
      close(jobs.size());
}

}  // namespace mamr
