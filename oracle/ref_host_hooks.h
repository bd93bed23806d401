/*
 * ref_host_hooks.h -- included by the extracted reference code (ref_kernels.inc) right after
 * its reference-tile loader, renamed readImageIntoSharedMemory_block (patchMatch.cu:620-667).
 * TEST INFRASTRUCTURE ONLY.
 *
 * On the GPU a block of 32 threads is one warp, and every thread loads its three columns of
 * the tile before any thread reads its neighbours' columns in computeNCC. The host runs the
 * block's threads as host threads, so the loader is fenced by two barriers: one before (every
 * thread is done with the previous row's tile) and one after (the whole tile is loaded).
 * Every thread of a block calls the loader the same number of times (patchMatch.cu:794,
 * :890, :1084 are outside the kernels' `col < width` tests), so the barriers always complete.
 */
template <int WINDOWSIZES>
inline void readImageIntoSharedMemory(float *refImg_I, int row, int col, const int &threadId, const bool &isRotated)
{
    pmr_block_barrier();
    readImageIntoSharedMemory_block<WINDOWSIZES>(refImg_I, row, col, threadId, isRotated);
    pmr_block_barrier();
}
