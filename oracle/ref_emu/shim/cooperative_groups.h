/* Host stand-in for <cooperative_groups.h> used by the CPU emulation of the
 * reference kernels (oracle/ref_emu).  Threads of a block run one after
 * another in increasing threadIdx order, so a block barrier is a no-op for
 * kernels whose threads only read shared values written by lower threads
 * (true of reorderDataAndFindCellStartD). */
#ifndef NW_EMU_COOPERATIVE_GROUPS_H
#define NW_EMU_COOPERATIVE_GROUPS_H
namespace cooperative_groups {
struct thread_block {};
inline thread_block this_thread_block() { return thread_block(); }
inline void sync(const thread_block&) {}
}
#endif
