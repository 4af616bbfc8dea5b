// The AMR driver: a whole miniAMR run on one rank through the mamr_* ABI
// (mamr_amr_run, include/miniamr_gb300.h).
//
// The host side of refinement lives here, with its own data structures: the
// per-slot block records, the parent records and the split and
// consolidation bookkeeping of the reference (ref/block.c:41-608) --
// slot allocation, parent records, block numbers, centres and the neighbour
// tables, kept exactly as the reference keeps them, stale entries of a
// reused slot included, because the next marking, the exchange and the
// reference's own mesh hash read them.  The marking runs on the device
// (mamr_mark_refine), the cell data movement too (mamr_split,
// mamr_consolidate), and each stretch of timesteps between refinements is
// one mamr_run_timesteps call.  Only public ABI calls are made, so the same
// source runs over the GPU library and over the CPU oracle.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "miniamr_gb300.h"

extern "C" int mamr_driver_fail(int code, const char *msg);

namespace {

// Errors carry a message to mamr_last_error through a status the caller
// turns into a return value.
struct Fail {
   int code;
   std::string msg;
};

struct Blk {
   long long number = -1;
   int level = 0, parent = -1, child_number = 0;
   int nei_level[6] = {0, 0, 0, 0, 0, 0};
   int nei[6][2][2] = {};
   int cen[3] = {0, 0, 0};
};

struct Par {
   long long number = -1;
   int level = 0, parent = -1, child_number = 0, refine = 0;
   int child[8] = {};
   int cen[3] = {0, 0, 0};
};

// Octant (i1 + 2*j1 + 4*k1) of the child that touches face c (W,E,S,N,D,U)
// at tangential position (a, b) of nei[c][a][b]: for x faces a runs along z
// and b along y; for y faces a along z, b along x; for z faces a along y,
// b along x (the quarter offsets of ref/comm.c:1613-1614,1645-1646,1674).
int face_child(int c, int a, int b)
{
   const int hi = c % 2;
   int i1, j1, k1;
   switch (c / 2) {
   case 0: i1 = hi; j1 = b; k1 = a; break;
   case 1: j1 = hi; i1 = b; k1 = a; break;
   default: k1 = hi; i1 = b; j1 = a; break;
   }
   return i1 + 2 * j1 + 4 * k1;
}

// Threads of the bookkeeping's list building (marking lists, meshes).
constexpr int kBookThreads = 4;

class Mesh {
 public:
   Mesh(int ix, int iy, int iz, int num_refine, int max_blocks)
      : ix_(ix), iy_(iy), iz_(iz), nr_(num_refine), cap_(max_blocks),
        b_(max_blocks), p_(max_blocks), start_(num_refine + 2, 0),
        count_(num_refine + 1, 0), used_(((size_t) max_blocks + 63) / 64, 0)
   {
      long long n = (long long) ix * iy * iz;
      for (int l = 1; l <= num_refine + 1; l++) {
         start_[l] = start_[l - 1] + n;
         n *= 8;
      }
   }

   // The initial lattice of init() on one rank (ref/init.c:453-560): slot
   // == block number, x fastest, level 0, lattice neighbours, -2 on the
   // domain boundary; centres i*size + size/2 with size = 2^(num_refine+1).
   void init()
   {
      const int n0 = ix_ * iy_ * iz_;
      if (n0 > cap_)
         throw Fail{MAMR_EINVAL, "max_blocks is smaller than the initial "
                                 "lattice"};
      const int size = 1 << (nr_ + 1);
      for (int k = 0, n = 0; k < iz_; k++)
         for (int j = 0; j < iy_; j++)
            for (int i = 0; i < ix_; i++, n++) {
               Blk &bp = b_[n];
               bp.number = n;
               occupy(n);
               bp.level = 0;
               bp.parent = -1;
               bp.child_number = 0;
               bp.cen[0] = i * size + size / 2;
               bp.cen[1] = j * size + size / 2;
               bp.cen[2] = k * size + size / 2;
               const int pos[3] = {i, j, k}, dim[3] = {ix_, iy_, iz_};
               const int step[3] = {1, ix_, ix_ * iy_};
               for (int c = 0; c < 6; c++) {
                  const int ax = c / 2, hi = c % 2;
                  const bool edge = hi ? pos[ax] == dim[ax] - 1 : pos[ax] == 0;
                  bp.nei_level[c] = edge ? -2 : 0;
                  bp.nei[c][0][0] = edge ? 0 : n + (hi ? step[ax] : -step[ax]);
               }
            }
      max_block_ = n0;
      active_ = n0;
      count_[0] = n0;
      pfree_ = 0;
   }

   int cur_max_level() const
   {
      for (int l = nr_; l >= 0; l--)
         if (count_[l])
            return l;
      return 0;
   }
   int active() const { return active_; }

   // Active slots in sorted_list order: level ascending, block number
   // descending (ref/block.c:610-625).  Level l's numbers fill
   // [start_[l], start_[l+1]), so start_[l] + start_[l+1] - 1 - number
   // orders the blocks that way within [0, start_[num_refine+1]); while
   // that range fits 32 bits the keys are radix-sorted (11 bits a pass),
   // else sorted as (level, complement of the number) pairs.
   std::vector<int> sorted() const
   {
      const long long total = start_[nr_ + 1];
      if (total > 0 && total <= (1ll << 32)) {
         // the keys of the active slots, word by word as mark_lists
         const int nw = (max_block_ + 63) / 64;
         std::vector<int> at(nw + 1, 0);
         for (int w = 0; w < nw; w++)
            at[w + 1] = at[w] + __builtin_popcountll(used_[w]);
         std::vector<uint32_t> k(at[nw]), k2;
         std::vector<int> v(at[nw]), v2;
#pragma omp parallel for num_threads(kBookThreads) schedule(static) \
   if (nw >= 256)
         for (int w = 0; w < nw; w++) {
            int q = at[w];
            for (uint64_t bits = used_[w]; bits; bits &= bits - 1) {
               const int n = w * 64 + __builtin_ctzll(bits);
               const Blk &bp = b_[n];
               k[q] = (uint32_t) (start_[bp.level] + start_[bp.level + 1] -
                                  1 - bp.number);
               v[q++] = n;
            }
         }
         k2.resize(k.size());
         v2.resize(v.size());
         int bits = 0;
         while (bits < 33 && (1ll << bits) < total)
            bits++;
         for (int sh = 0; sh < bits; sh += 11) {
            size_t cnt[2049] = {};
            for (const uint32_t x : k)
               cnt[((x >> sh) & 2047) + 1]++;
            for (int d = 0; d < 2048; d++)
               cnt[d + 1] += cnt[d];
            for (size_t q = 0; q < k.size(); q++) {
               const size_t to = cnt[(k[q] >> sh) & 2047]++;
               k2[to] = k[q];
               v2[to] = v[q];
            }
            k.swap(k2);
            v.swap(v2);
         }
         return v;
      }
      // one key per block, level in the high bits and the complement of
      // the number below it (numbers < 2^58: init blocks x 8^num_refine
      // with num_refine <= 20 stays far below that for any lattice that
      // fits a pool)
      std::vector<std::pair<uint64_t, int>> k;
      k.reserve(active_);
      for (int n = 0; n < max_block_; n++)
         if (b_[n].number >= 0)
            k.emplace_back(((uint64_t) b_[n].level << 58) |
                              (((uint64_t) 1 << 58) - 1 -
                               (uint64_t) b_[n].number),
                           n);
      std::sort(k.begin(), k.end());
      std::vector<int> s(k.size());
      for (size_t q = 0; q < k.size(); q++)
         s[q] = k[q].second;
      return s;
   }

   void export_mesh(std::vector<mamr_block> &mesh,
                    std::vector<int64_t> &numbers, std::vector<int32_t> &cen)
      const
   {
      const std::vector<int> s = sorted();
      mesh.resize(s.size());
      numbers.resize(s.size());
      cen.resize(3 * s.size());
      const long long ns = (long long) s.size();
#pragma omp parallel for num_threads(kBookThreads) schedule(static) \
   if (ns >= 16384)
      for (long long q = 0; q < ns; q++) {
         const Blk &bp = b_[s[q]];
         mamr_block &m = mesh[q];
         m.slot = s[q];
         m.level = bp.level;
         for (int c = 0; c < 6; c++) {
            m.nei_level[c] = bp.nei_level[c];
            for (int a = 0; a < 2; a++)
               for (int d = 0; d < 2; d++)
                  m.nei[c][a][d] = bp.nei[c][a][d];
         }
         numbers[q] = bp.number;
         for (int d = 0; d < 3; d++)
            cen[3 * q + d] = bp.cen[d];
      }
   }

   // The marking's inputs (ref/block.h: the active blocks -- in slot
   // order, since the marking's result does not depend on the order --
   // and parents [0, max_active_parent)) and, afterwards, its flags back.
   void mark_lists(std::vector<mamr_mark_block> &mb,
                   std::vector<mamr_mark_parent> &pa) const
   {
      // the active slots word by word (the occupancy bitmap), each word's
      // first list position from the counts before it, so that the words
      // fill their stretches of the list on several threads
      const int nw = (max_block_ + 63) / 64;
      std::vector<int> at(nw + 1, 0);
      for (int w = 0; w < nw; w++)
         at[w + 1] = at[w] + __builtin_popcountll(used_[w]);
      mb.resize(at[nw]);
#pragma omp parallel for num_threads(kBookThreads) schedule(static) \
   if (nw >= 256)
      for (int w = 0; w < nw; w++) {
         int q = at[w];
         for (uint64_t bits = used_[w]; bits; bits &= bits - 1) {
            const int n = w * 64 + __builtin_ctzll(bits);
            const Blk &bp = b_[n];
            mamr_mark_block &m = mb[q++];
            m.slot = n;
            m.level = bp.level;
            m.parent = bp.parent;
            for (int d = 0; d < 3; d++)
               m.cen[d] = bp.cen[d];
            for (int c = 0; c < 6; c++) {
               m.nei_level[c] = bp.nei_level[c];
               m.nei[c] = bp.nei[c][0][0];
            }
         }
      }
      pa.resize(max_parent_);
#pragma omp parallel for num_threads(kBookThreads) schedule(static) \
   if (max_parent_ >= 4096)
      for (int p = 0; p < max_parent_; p++) {
         pa[p].active = p_[p].number >= 0;
         for (int o = 0; o < 8; o++)
            pa[p].child[o] = p_[p].child[o];
      }
   }
   // The marking's flags: the blocks to split (by level, in slot order --
   // mb lists the blocks in slot order) and the parents' flags.
   void set_flags(const std::vector<mamr_mark_block> &mb,
                  const std::vector<int32_t> &bref,
                  const std::vector<int32_t> &pref)
   {
      marked_.resize(nr_ + 1);
      for (std::vector<int> &m : marked_)
         m.clear();
      for (size_t q = 0; q < mb.size(); q++)
         if (bref[q] == 1 && mb[q].level <= nr_)
            marked_[mb[q].level].push_back(mb[q].slot);
      // and the parents to consolidate, by level in record order (split
      // adds records with flag 0 and changes no other record's flag, level
      // or activity, so consolidate's scan of the records finds these)
      coarsen_.resize(nr_ + 1);
      for (std::vector<int> &m : coarsen_)
         m.clear();
      for (int p = 0; p < max_parent_; p++)
         if (p_[p].number >= 0) {
            p_[p].refine = pref[p];
            if (pref[p] == -1 && p_[p].level <= nr_)
               coarsen_[p_[p].level].push_back(p);
         }
   }

   // split_blocks() (ref/block.c:41-343) on one rank: levels ascending,
   // blocks in slot order; each refined block gets a parent record (the
   // first unused one) and eight children, each in the first free slot at
   // or after a running index that also falls back to a freed parent's
   // slot; numbers, centres and neighbour tables as the reference's.
   void split(std::vector<mamr_split_job> &jobs)
   {
      jobs.clear();
      const int top = cur_max_level();
      // the blocks marked to split, by level in slot order (set_flags):
      // splitting one level adds children in free slots and moves no other
      // block, so the reference's slot scan of each level finds these
      int m = 0;
      for (int level = 0; level <= top && level < (int) marked_.size();
           level++) {
         for (const int n : marked_[level]) {
            Blk &bp = b_[n];
            const long long nl = bp.number - start_[level];
            const long long lx = (long long) ix_ << level,
                            ly = (long long) iy_ << level;
            const long long zp = nl / (lx * ly), yp = (nl % (lx * ly)) / lx,
                            xp = nl % lx;
            if (active_ + 8 > cap_)
               throw Fail{MAMR_ENOMEM, "split: more blocks needed than "
                                       "max_blocks"};
            active_ += 7;
            count_[level]--;
            count_[level + 1] += 8;
            // the first unused parent record (every record below pfree_
            // is in use)
            int p = pfree_;
            while (p < max_parent_ && p_[p].number >= 0)
               p++;
            if (p == cap_)
               throw Fail{MAMR_ENOMEM, "split: more parent records needed"};
            if (p == max_parent_)
               max_parent_++;
            pfree_ = p + 1;
            Par &pp = p_[p];
            pp.number = bp.number;
            pp.level = bp.level;
            pp.parent = bp.parent;
            pp.child_number = bp.child_number;
            if (pp.parent >= 0)
               p_[pp.parent].child[pp.child_number] = -1 - p;
            pp.refine = 0;
            for (int d = 0; d < 3; d++)
               pp.cen[d] = bp.cen[d];
            mamr_split_job job;
            job.parent = n;
            int sib[8];
            const int half = 1 << (nr_ - level - 1);
            const long long cx = (long long) ix_ << (level + 1),
                            cy = (long long) iy_ << (level + 1);
            for (int o = 0; o < 8; o++) {
               m = next_free(m);
               if (m == cap_)
                  throw Fail{MAMR_ENOMEM, "split: no inactive block slot"};
               max_block_ = std::max(max_block_, m + 1);
               Blk &c = b_[m];
               occupy(m);
               sib[o] = m;
               pp.child[o] = m;
               job.child[o] = m;
               c.level = level + 1;
               c.parent = p;
               c.child_number = o;
               const int i1 = o % 2, j1 = (o / 2) % 2, k1 = o / 4;
               c.number = ((2 * zp + k1) * cy + (2 * yp + j1)) * cx +
                          2 * xp + i1 + start_[level + 1];
               c.cen[0] = bp.cen[0] + (2 * i1 - 1) * half;
               c.cen[1] = bp.cen[1] + (2 * j1 - 1) * half;
               c.cen[2] = bp.cen[2] + (2 * k1 - 1) * half;
            }
            jobs.push_back(job);
            for (int c = 0; c < 6; c++) {
               const int opp = c ^ 1, bit = 1 << (c / 2);
               // siblings facing each other across the parent's mid-plane
               for (int a = 0; a < 2; a++)
                  for (int d = 0; d < 2; d++) {
                     const int s = face_child(c, a, d);
                     b_[sib[s ^ bit]].nei_level[c] = level + 1;
                     b_[sib[s ^ bit]].nei[c][0][0] = sib[s];
                  }
               // the children on face c take over the parent's neighbour
               const int nlv = bp.nei_level[c];
               if (nlv == -2) {
                  for (int a = 0; a < 2; a++)
                     for (int d = 0; d < 2; d++) {
                        Blk &ch = b_[sib[face_child(c, a, d)]];
                        ch.nei_level[c] = -2;
                        ch.nei[c][0][0] = 0;
                     }
               } else if (nlv == level) {
                  const int other = bp.nei[c][0][0];
                  b_[other].nei_level[opp] = level + 1;
                  for (int a = 0; a < 2; a++)
                     for (int d = 0; d < 2; d++) {
                        const int ch = sib[face_child(c, a, d)];
                        b_[ch].nei_level[c] = level;
                        b_[ch].nei[c][0][0] = other;
                        b_[other].nei[opp][a][d] = ch;
                     }
               } else if (nlv == level + 1) {
                  for (int a = 0; a < 2; a++)
                     for (int d = 0; d < 2; d++) {
                        const int other = bp.nei[c][a][d];
                        const int ch = sib[face_child(c, a, d)];
                        b_[ch].nei_level[c] = level + 1;
                        b_[ch].nei[c][0][0] = other;
                        b_[other].nei_level[opp] = level + 1;
                        b_[other].nei[opp][0][0] = ch;
                     }
               } else {
                  // a coarser neighbour would have to split first: the
                  // marking's rules exclude it on one rank
                  throw Fail{MAMR_EMESH, "split: misconnected block"};
               }
            }
            // the parent's slot is free again and may take a later child
            bp.number = -1;
            release(n);
            if (n < m)
               m = n;
         }
      }
   }

   // consolidate_blocks() (ref/block.c:349-608) on one rank: levels
   // descending, parent records in order; each parent marked -1 becomes a
   // block again in the first free slot from 0, its eight children freed,
   // the neighbour tables rewired as the reference's.
   void consolidate(std::vector<mamr_consolidate_job> &jobs)
   {
      jobs.clear();
      for (int level = std::min(cur_max_level(), (int) coarsen_.size() - 1);
           level >= 0; level--)
         for (const int p : coarsen_[level]) {
            Par &pp = p_[p];
            if (pp.number < 0 || pp.level != level || pp.refine != -1)
               continue;
            // the first free slot
            const int n = next_free(0);
            if (n == cap_)
               throw Fail{MAMR_ENOMEM, "consolidate: no free block slot"};
            max_block_ = std::max(max_block_, n + 1);
            active_ -= 7;
            count_[level]++;
            count_[level + 1] -= 8;
            Blk &bp = b_[n];
            bp.number = pp.number;
            occupy(n);
            pp.number = -1;
            pfree_ = std::min(pfree_, p);
            bp.level = pp.level;
            bp.parent = pp.parent;
            bp.child_number = pp.child_number;
            if (bp.level)
               p_[bp.parent].child[bp.child_number] = n;
            for (int d = 0; d < 3; d++)
               bp.cen[d] = pp.cen[d];
            mamr_consolidate_job job;
            job.target = n;
            for (int o = 0; o < 8; o++) {
               b_[pp.child[o]].number = -1;
               release(pp.child[o]);
               job.child[o] = pp.child[o];
            }
            jobs.push_back(job);
            for (int c = 0; c < 6; c++) {
               const int opp = c ^ 1;
               const Blk &first = b_[pp.child[face_child(c, 0, 0)]];
               if (first.nei_level[c] == -2) {
                  bp.nei_level[c] = -2;
               } else if (first.nei_level[c] == level) {
                  const int nb = first.nei[c][0][0];
                  bp.nei[c][0][0] = nb;
                  bp.nei_level[c] = level;
                  b_[nb].nei[opp][0][0] = n;
                  b_[nb].nei_level[opp] = level;
               } else {
                  for (int a = 0; a < 2; a++)
                     for (int d = 0; d < 2; d++) {
                        const Blk &ch = b_[pp.child[face_child(c, a, d)]];
                        const int nb = ch.nei[c][0][0];
                        if (ch.nei_level[c] == level + 2)
                           throw Fail{MAMR_EMESH, "consolidate: neighbour "
                                                  "two levels finer"};
                        bp.nei[c][a][d] = nb;
                        bp.nei_level[c] = level + 1;
                        b_[nb].nei[opp][0][0] = n;
                        b_[nb].nei_level[opp] = level;
                     }
               }
            }
         }
   }

 private:
   int ix_, iy_, iz_, nr_, cap_;
   std::vector<Blk> b_;
   std::vector<Par> p_;
   std::vector<long long> start_;
   std::vector<long long> count_;
   int max_block_ = 0, max_parent_ = 0, active_ = 0;
   // a lower bound of the first unused parent record: the search the
   // reference starts from 0 starts here, with the same result
   int pfree_ = 0;
   // one bit per slot, set while the slot holds a block: the reference's
   // scans for the next free slot (from a running index in split, from 0 in
   // consolidate) skip 64 slots a word
   std::vector<uint64_t> used_;
   std::vector<std::vector<int>> marked_;   // slots to split, by level
   std::vector<std::vector<int>> coarsen_;  // parents to consolidate

   void occupy(int n) { used_[n >> 6] |= (uint64_t) 1 << (n & 63); }
   void release(int n) { used_[n >> 6] &= ~((uint64_t) 1 << (n & 63)); }
   // The first free slot at or after n, cap_ if none.
   int next_free(int n) const
   {
      if (n >= cap_)
         return cap_;
      size_t w = (size_t) n >> 6;
      uint64_t free_bits = ~used_[w] & (~(uint64_t) 0 << (n & 63));
      while (!free_bits) {
         if (++w == used_.size())
            return cap_;
         free_bits = ~used_[w];
      }
      const int f = (int) (w * 64) + __builtin_ctzll(free_bits);
      return f < cap_ ? f : cap_;
   }
};

// move() (ref/move.c:37-63): position and size advance by delta; with
// bounce 1 the centre reflects off the unit cube's faces and the motion
// reverses.  The reference's bounce-2 branch hangs off the inner if-chain
// of the bounce-1 branch (C's dangling else) and can never run, so any
// other bounce value only moves the object.
void move(std::vector<mamr_amr_object> &objs, double delta)
{
   for (mamr_amr_object &o : objs)
      for (int d = 0; d < 3; d++) {
         o.cen[d] += delta * o.move[d];
         o.size[d] += delta * o.inc[d];
         if (o.bounce != 1)
            continue;
         if (o.cen[d] >= 1.0) {
            o.cen[d] = 2.0 - o.cen[d];
            o.move[d] = -o.move[d];
         } else if (o.cen[d] <= 0.0) {
            o.cen[d] = 0.0 - o.cen[d];
            o.move[d] = -o.move[d];
         }
      }
}

void check(int r, const char *what)
{
   if (r != MAMR_OK)
      throw Fail{r, std::string(what) + ": " + mamr_last_error()};
}

double now()
{
   return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Seconds since t; t moves to now.
double lap(double &t)
{
   const double n = now(), d = n - t;
   t = n;
   return d;
}

// One refinement as the stages see it: the split and consolidation job
// lists of its steps in order, then the mesh it leaves.
struct Plan {
   int ts = 0;
   std::vector<std::vector<mamr_split_job>> split;
   std::vector<std::vector<mamr_consolidate_job>> cons;
   std::vector<mamr_block> mesh;
   std::vector<int64_t> numbers;
   std::vector<int32_t> cen;
   int active = 0;
};

// The refinement side of the run: the octree bookkeeping and the marking,
// on a thread of its own.  Nothing it computes depends on cell values --
// the marking reads the mesh and the objects, the objects move by their
// own arithmetic -- so it runs ahead of the stages and hands each
// refinement over as a Plan through a short queue; the stage side applies
// them in order.  The marking goes through a context of its own (one
// variable), so that its device work does not wait behind the stages.
class Planner {
 public:
   Planner(mamr_ctx *mctx, const mamr_amr_params &p,
           const std::vector<mamr_amr_object> &objs, int cap)
      : mctx_(mctx), prm_(p), objs_(objs),
        mesh_(p.init_x, p.init_y, p.init_z, p.num_refine, cap)
   {
      mesh_.init();
   }
   ~Planner() { stop(); }

   // The initial lattice's mesh (before the thread starts).
   void initial(Plan &out) const
   {
      mesh_.export_mesh(out.mesh, out.numbers, out.cen);
      out.active = mesh_.active();
   }

   void start()
   {
      th_ = std::thread([this] { body(); });
   }

   // The next refinement, in order; false once the planner has none left.
   bool pop(Plan &out)
   {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [this] { return !q_.empty() || done_; });
      if (q_.empty()) {
         if (err_)
            throw Fail{err_, err_msg_};
         return false;
      }
      out = std::move(q_.front());
      q_.pop_front();
      cv_.notify_all();
      return true;
   }

   void stop()
   {
      {
         std::lock_guard<std::mutex> lk(mu_);
         stop_ = true;
      }
      cv_.notify_all();
      if (th_.joinable())
         th_.join();
   }

   double mark_s = 0.0, book_s = 0.0;
   int marking_steps = 0;

 private:
   static constexpr size_t kAhead = 3;   // refinements planned ahead

   void push(Plan &&p)
   {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [this] { return q_.size() < kAhead || stop_; });
      if (stop_)
         throw Fail{MAMR_OK, ""};
      q_.push_back(std::move(p));
      cv_.notify_all();
   }

   void body()
   {
      try {
         if (prm_.num_refine || prm_.uniform_refine)
            refine(0);
         // ref/driver.c:110-117: move() every timestep, refine() every
         // refine_freq timesteps
         if (prm_.num_refine && !prm_.uniform_refine) {
            const int n_ts = std::max(1, prm_.num_tsteps);
            for (int ts = 1; ts <= n_ts; ts++) {
               move(objs_, 1.0);
               if (!(ts % prm_.refine_freq))
                  refine(ts);
            }
         }
      } catch (const Fail &f) {
         std::lock_guard<std::mutex> lk(mu_);
         if (f.code != MAMR_OK) {
            err_ = f.code;
            err_msg_ = f.msg;
         }
      } catch (const std::bad_alloc &) {
         std::lock_guard<std::mutex> lk(mu_);
         err_ = MAMR_ENOMEM;
         err_msg_ = "host allocation";
      }
      std::lock_guard<std::mutex> lk(mu_);
      done_ = true;
      cv_.notify_all();
   }

   // refine(ts) (ref/refine.c:38-210) on one rank: num_refine steps at
   // ts 0, block_change steps after, each the marking, the splits and the
   // consolidations.
   void refine(int ts)
   {
      Plan plan = recycled();
      plan.ts = ts;
      plan.split.clear();
      plan.cons.clear();
      const int steps = ts ? (prm_.block_change ? prm_.block_change
                                                : prm_.num_refine)
                           : prm_.num_refine;
      std::vector<mamr_mark_block> &mb = mb_;
      std::vector<mamr_mark_parent> &pa = pa_;
      std::vector<int32_t> &bref = bref_, &pref = pref_;
      std::vector<mamr_object> mo(objs_.size());
      mamr_mark_params mp;
      memset(&mp, 0, sizeof(mp));
      mp.num_refine = prm_.num_refine;
      mp.refine_ghost = prm_.refine_ghost;
      mp.uniform_refine = prm_.uniform_refine;
      const int size = 1 << (prm_.num_refine + 1);
      mp.mesh_size[0] = prm_.init_x * size;
      mp.mesh_size[1] = prm_.init_y * size;
      mp.mesh_size[2] = prm_.init_z * size;
      for (int i = 0; i < steps; i++) {
         double t = now();
         for (size_t o = 0; o < objs_.size(); o++) {
            mo[o].type = objs_[o].type;
            mo[o].reserved = 0;
            for (int d = 0; d < 3; d++) {
               mo[o].cen[d] = objs_[o].cen[d];
               mo[o].size[d] = objs_[o].size[d];
            }
         }
         mesh_.mark_lists(mb, pa);
         bref.assign(mb.size() + 1, 0);
         pref.assign(pa.size() + 1, 0);
         book_s += lap(t);
         check(mamr_mark_refine(mctx_, &mp,
                                prm_.uniform_refine ? nullptr : mo.data(),
                                prm_.uniform_refine ? 0
                                                    : (int32_t) mo.size(),
                                mb.data(), (int32_t) mb.size(), pa.data(),
                                (int32_t) pa.size(), bref.data(),
                                pref.data()),
               "mamr_mark_refine");
         mark_s += lap(t);
         marking_steps++;
         mesh_.set_flags(mb, bref, pref);
         plan.split.emplace_back();
         plan.cons.emplace_back();
         mesh_.split(plan.split.back());
         mesh_.consolidate(plan.cons.back());
         book_s += lap(t);
         // a step that changed nothing leaves the marking's inputs as they
         // were (it starts from reset flags, and the objects move only
         // between refinements), so the remaining steps change nothing
         // either
         if (plan.split.back().empty() && plan.cons.back().empty())
            break;
      }
      double t = now();
      mesh_.export_mesh(plan.mesh, plan.numbers, plan.cen);
      plan.active = mesh_.active();
      book_s += lap(t);
      push(std::move(plan));
   }

   // A used plan back from the stage side (its buffers keep their
   // capacity), or a new one.
   Plan recycled()
   {
      std::lock_guard<std::mutex> lk(mu_);
      if (free_.empty())
         return Plan();
      Plan p = std::move(free_.back());
      free_.pop_back();
      return p;
   }

 public:
   // The stage side hands an applied plan back for reuse.
   void give_back(Plan &&p)
   {
      std::lock_guard<std::mutex> lk(mu_);
      if (free_.size() < kAhead + 1)
         free_.push_back(std::move(p));
   }

 private:
   mamr_ctx *mctx_;
   const mamr_amr_params &prm_;
   std::vector<mamr_amr_object> objs_;
   Mesh mesh_;
   std::vector<mamr_mark_block> mb_;
   std::vector<mamr_mark_parent> pa_;
   std::vector<int32_t> bref_, pref_;
   std::vector<Plan> free_;
   std::thread th_;
   std::mutex mu_;
   std::condition_variable cv_;
   std::deque<Plan> q_;
   bool done_ = false, stop_ = false;
   int err_ = MAMR_OK;
   std::string err_msg_;
};

// The stage side: the cell data, the stages and each refinement's data
// movement and mesh, in the reference driver's order.
struct Run {
   mamr_ctx *ctx;
   const mamr_config &cfg;
   const mamr_amr_params &prm;
   std::vector<mamr_amr_object> objs;
   double *sums;
   int64_t max_sums, n_sums = 0;
   mamr_amr_event event;
   void *user;
   mamr_amr_stats st{};
   int flags;    // the stretches' run flags (batched until it is refused)
   int active = 0;
   double ev_s = 0.0;   // time spent in the caller's event callback, which
                        // the stats leave out

   void emit(int kind, int ts, const void *data, int32_t n,
             const int64_t *numbers, const int32_t *cen)
   {
      if (!event)
         return;
      const double a = now();
      event(user, kind, ts, data, n, numbers, cen);
      ev_s += now() - a;
   }

   Run(mamr_ctx *c, const mamr_config &cf, const mamr_amr_params &p)
      : ctx(c), cfg(cf), prm(p), flags(p.run_flags & ~MAMR_RUN_NO_GHOSTS)
   {
   }

   void put_sums(const double *s, int64_t n)
   {
      for (int64_t q = 0; q < n && n_sums < max_sums; q++)
         sums[n_sums++] = s[q];
   }

   void set_mesh(const Plan &p)
   {
      check(mamr_set_mesh(ctx, p.mesh.data(), (int32_t) p.mesh.size()),
            "mamr_set_mesh");
      active = p.active;
      st.max_active = std::max(st.max_active, (int32_t) p.mesh.size());
   }

   // One refinement from the planner: its job lists, then its mesh.
   void apply(Planner &pl)
   {
      const double t0 = now(), ev0 = ev_s;
      Plan p;
      if (!pl.pop(p))
         throw Fail{MAMR_EINVAL, "refinement plan missing"};
      double t = now();
      st.wait_seconds += t - t0;
      for (size_t i = 0; i < p.split.size(); i++) {
         if (!p.split[i].empty()) {
            check(mamr_split(ctx, p.split[i].data(),
                             (int32_t) p.split[i].size()),
                  "mamr_split");
            st.data_seconds += lap(t);
            emit(1, p.ts, p.split[i].data(), (int32_t) p.split[i].size(),
                 nullptr, nullptr);
            t = now();
         }
         if (!p.cons[i].empty()) {
            check(mamr_consolidate(ctx, p.cons[i].data(),
                                   (int32_t) p.cons[i].size()),
                  "mamr_consolidate");
            st.data_seconds += lap(t);
            emit(2, p.ts, p.cons[i].data(), (int32_t) p.cons[i].size(),
                 nullptr, nullptr);
            t = now();
         }
      }
      // queued behind the data movement on the same stream
      set_mesh(p);
      st.mesh_seconds += lap(t);
      // the refinement's device work (cell movement, mesh upload) done
      // here, so that the stage stretches' time holds only stages
      check(mamr_sync(ctx), "mamr_sync");
      st.data_seconds += lap(t);
      emit(3, p.ts, p.mesh.data(), (int32_t) p.mesh.size(), p.numbers.data(),
           p.cen.data());
      st.refinements++;
      pl.give_back(std::move(p));
      st.refine_seconds += now() - t0 - (ev_s - ev0);
   }

   // A stretch of n_ts timesteps.  Batched 7-point stretches before the
   // last leave the ghost cells in the pool as they were: the next
   // stretch gathers its ghosts from the interiors, and splits and
   // consolidations move interiors only, so only the last stretch's
   // ghost layer (the one the reference's last exchange leaves) is
   // written back.
   void stages(int n_ts, int first_stage, bool final)
   {
      if (n_ts <= 0)
         return;
      const int V = cfg.num_vars, spt = prm.stages_per_ts;
      int per_ts = 0;
      if (prm.checksum_freq)
         for (int s = 0; s < spt; s++)
            per_ts += !(s % prm.checksum_freq);
      std::vector<double> s((size_t) std::max(1, per_ts * n_ts) * V);
      int32_t got = 0;
      const double t0 = now();
      const int fl = (flags & MAMR_RUN_BATCHED) && cfg.stencil == 7 && !final
                        ? flags | MAMR_RUN_NO_GHOSTS
                        : flags;
      int r = mamr_run_timesteps(ctx, n_ts, spt, prm.checksum_freq,
                                 first_stage, fl, s.data(), &got);
      if (r == MAMR_EUNSUP && (flags & MAMR_RUN_BATCHED)) {
         // refused before any stage ran: the plain path from here on
         flags = MAMR_RUN_PLAIN;
         r = mamr_run_timesteps(ctx, n_ts, spt, prm.checksum_freq,
                                first_stage, flags, s.data(), &got);
      }
      check(r, "mamr_run_timesteps");
      st.stretches++;
      st.plain_stretches += (prm.run_flags & MAMR_RUN_BATCHED) &&
                            !(flags & MAMR_RUN_BATCHED);
      check(mamr_sync(ctx), "mamr_sync");
      st.stage_seconds += now() - t0;
      put_sums(s.data(), (int64_t) got * V);
      st.updates += (int64_t) n_ts * spt * active *
                    ((int64_t) cfg.nx * cfg.ny * cfg.nz) * V;
   }

   void run(mamr_ctx *mctx)
   {
      const double t0 = now();
      const int V = cfg.num_vars;
      if (cfg.stencil == 0) {
         double a1 = 0.0;
         std::vector<double> a0((size_t) std::max(1, V / 4));
         check(mamr_work_coefficients(V, &a1, a0.data()),
               "mamr_work_coefficients");
         check(mamr_set_work_params(ctx, a1, a0.data(), V / 4),
               "mamr_set_work_params");
      }
      Planner pl(mctx, prm, objs, cfg.max_blocks);
      // init(): the lattice, its values (one rand() stream over all the
      // initial blocks, so generated at once) and their checksums
      const int n0 = prm.init_x * prm.init_y * prm.init_z;
      {
         const size_t per = (size_t) V * (cfg.nx + 2) * (cfg.ny + 2) *
                            (cfg.nz + 2);
         std::vector<double> all((size_t) n0 * per);
         check(mamr_initial_values(&cfg, n0, all.data()),
               "mamr_initial_values");
         std::vector<int32_t> slots(n0);
         for (int q = 0; q < n0; q++)
            slots[q] = q;
         check(mamr_upload_blocks(ctx, slots.data(), n0, all.data()),
               "mamr_upload_blocks");
      }
      {
         Plan init;
         pl.initial(init);
         set_mesh(init);
      }
      pl.start();
      for (int var = 0; var < V; var++) {
         double s = 0.0;
         check(mamr_check_sum(ctx, var, &s), "mamr_check_sum");
         put_sums(&s, 1);
      }
      if (prm.num_refine || prm.uniform_refine)
         apply(pl);
      // ref/driver.c:66-140: stages, move, refine every refine_freq; the
      // loop tests for the end after the first timestep, so it runs at
      // least one
      const bool moving = prm.num_refine && !prm.uniform_refine;
      const int n_ts = std::max(1, prm.num_tsteps);
      int pending = 0, first_ts = 1;
      for (int ts = 1; ts <= n_ts; ts++) {
         pending++;
         const bool refine_now = moving && !(ts % prm.refine_freq);
         if (refine_now || ts == n_ts) {
            stages(pending, (first_ts - 1) * prm.stages_per_ts, ts == n_ts);
            first_ts = ts + 1;
            pending = 0;
         }
         if (refine_now)
            apply(pl);
      }
      pl.stop();
      st.mark_seconds = pl.mark_s;
      st.bookkeeping_seconds = pl.book_s;
      st.marking_steps = pl.marking_steps;
      check(mamr_sync(ctx), "mamr_sync");
      st.final_active = active;
      st.total_seconds = now() - t0 - ev_s;
   }
};

}  // namespace

extern "C" int mamr_amr_run(mamr_ctx *ctx, const mamr_config *cfg,
                            const mamr_amr_params *p,
                            const mamr_amr_object *objects, int32_t n_objects,
                            double *sums, int64_t max_sums, int64_t *n_sums,
                            mamr_amr_event event, void *user,
                            mamr_amr_stats *stats)
{
   if (!ctx || !cfg || !p || (n_objects && !objects) || n_objects < 0 ||
       (max_sums && !sums) || max_sums < 0)
      return mamr_driver_fail(MAMR_EINVAL, "mamr_amr_run: bad arguments");
   if (p->init_x < 1 || p->init_y < 1 || p->init_z < 1 ||
       p->num_refine < 0 || p->num_refine > 20 || p->block_change < 0 ||
       p->refine_freq < 1 || p->num_tsteps < 0 || p->stages_per_ts < 1 ||
       p->checksum_freq < 0)
      return mamr_driver_fail(MAMR_EINVAL, "mamr_amr_run: bad parameters");
   for (int r = 0; r < 8; r++)
      if (p->reserved[r])
         return mamr_driver_fail(MAMR_EINVAL, "mamr_amr_run: reserved "
                                              "parameters must be zero");
   Run run(ctx, *cfg, *p);
   run.objs.assign(objects, objects + n_objects);
   run.sums = sums;
   run.max_sums = max_sums;
   run.event = event;
   run.user = user;
   // the marking's own context: the block shape, one variable
   mamr_config mc = *cfg;
   mc.num_vars = 1;
   mc.stencil = cfg->stencil == 27 ? 27 : 7;
   mc.code = 0;
   mc.permute = 0;
   mamr_ctx *mctx = nullptr;
   int status = mamr_create(&mc, &mctx);
   if (status != MAMR_OK)
      return status;
   try {
      run.run(mctx);
   } catch (const Fail &f) {
      status = f.code;
      char buf[400];
      snprintf(buf, sizeof(buf), "mamr_amr_run: %s", f.msg.c_str());
      mamr_driver_fail(status, buf);
   } catch (const std::bad_alloc &) {
      status = MAMR_ENOMEM;
      mamr_driver_fail(status, "mamr_amr_run: host allocation");
   }
   mamr_destroy(mctx);
   if (n_sums)
      *n_sums = run.n_sums;
   if (stats)
      *stats = run.st;
   return status;
}
