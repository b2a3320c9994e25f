/* ss4d_slab.c — one volume split across ranks by frames (t-slabs), host side.
 *
 * The reference's MPI program (segmentation4D_mpi.c) gives every process a
 * slab of frames; _segTimeStep_mpi_ (:282-397) sweeps its slab's red voxels,
 * exchanges one ghost frame with each neighbour (_communication_mpi_,
 * :485-526, called at :330), sweeps the black voxels, exchanges again (:361),
 * and sums the residual over all processes every iteration (MPI_Allreduce,
 * :386) before the stop test.  This file holds what does not depend on where
 * the sweeps run: the partition of the frames and that loop, driven through
 * the caller's compute callbacks (ss4d_slab_ops) and communication callbacks
 * (ss4d_slab_comm).  The GPU's callbacks are in ss4d_api.cu.
 *
 * Red voxels are those with an even global index sum (i + j + k + l).  The
 * reference offsets l by N * rank with N = (lMax - 2) / processes (:289,
 * :307), which names the wrong voxels red whenever slabs are uneven.  Here
 * the partition gives every slab but the last an even number of frames, so
 * every slab starts on an even global frame offset and its local index sum
 * has the global parity: the red set is the global one on every rank. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "../../include/ss4d.h"

extern void ss4d_set_error_text_c(const char *msg);

static ss4d_status fail(ss4d_status st, const char *msg)
{
    ss4d_set_error_text_c(msg);
    return st;
}

ss4d_status ss4d_slab_partition(int nt, int nranks, int *first, int *count)
{
    if (!first || !count || nranks < 1 || nt < 1)
        return fail(SS4D_ERR_INVALID, "ss4d_slab_partition: invalid argument");
    if (nt < 2 * nranks - 1)
        return fail(SS4D_ERR_INVALID,
                    "ss4d_slab_partition: fewer than 2 frames per rank (every slab but the last needs an even count)");
    /* pairs of frames shared out as evenly as possible; the last slab takes
     * the odd frame, if any */
    const int pairs = nt / 2, odd = nt % 2;
    int f = 1;
    for (int r = 0; r < nranks; ++r) {
        int p = pairs / nranks + (r < pairs % nranks ? 1 : 0);
        int c = 2 * p + (r == nranks - 1 ? odd : 0);
        first[r] = f;
        count[r] = c;
        f += c;
    }
    /* with nt >= 2 nranks - 1 every slab holds a frame; checked all the same */
    for (int r = 0; r < nranks; ++r)
        if (count[r] < 1)
            return fail(SS4D_ERR_INVALID, "ss4d_slab_partition: a rank would hold no frame");
    return SS4D_OK;
}

ss4d_status ss4d_slab_sor_loop(const ss4d_slab_ops *ops, const ss4d_slab_comm *comm, const ss4d_params *p,
                               long long nint_global, ss4d_step_stats *stats)
{
    if (!ops || !comm || !p || !ops->half_sweep || !ops->residual || !comm->exchange || !comm->allreduce_sum ||
        !ops->u || ops->lMax < 3 || ops->frame_elems < 1 || nint_global < 1)
        return fail(SS4D_ERR_INVALID, "ss4d_slab_sor_loop: invalid argument");
    if (p->maxNoGSIteration < 1)
        return fail(SS4D_ERR_INVALID, "ss4d_slab_sor_loop: maxNoGSIteration must be >= 1");
    /* a sum of nint_global terms in another order than the reference's
     * serial loop differs from it by up to about nint * 2^-53 relative */
    const double band = fabs(p->gsTol) * (double)nint_global * 0x1p-53;
    double R = 0.0, R1 = 0.0;
    int z = 0, near = 0;
    do {
        z = z + 1;
        for (int colour = 0; colour < 2; ++colour) {
            if (ops->half_sweep(ops->ctx, colour))
                return fail(SS4D_ERR_CUDA, "ss4d_slab_sor_loop: a half-sweep failed");
            if (comm->exchange(comm->ctx, ops->u, ops->frame_elems, ops->lMax, ops->stream))
                return fail(SS4D_ERR_CUDA, "ss4d_slab_sor_loop: the ghost-frame exchange failed");
        }
        double part = 0.0;
        if (ops->residual(ops->ctx, &part))
            return fail(SS4D_ERR_CUDA, "ss4d_slab_sor_loop: the residual failed");
        R = part;
        if (comm->allreduce_sum(comm->ctx, &R))
            return fail(SS4D_ERR_CUDA, "ss4d_slab_sor_loop: the residual sum over ranks failed");
        if (z == 1)
            R1 = R;
        near |= fabs(R - p->gsTol) <= band;
    } while (R > p->gsTol && z < p->maxNoGSIteration);
    const ss4d_status st = isfinite(R) ? SS4D_OK : SS4D_ERR_NONFINITE;
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->iterations = z;
        stats->residual = R;
        stats->first_residual = R1;
        stats->near_tolerance = near;
        stats->status = st;
    }
    if (st != SS4D_OK)
        return fail(st, "ss4d_slab_sor_loop: the residual is not finite");
    return SS4D_OK;
}
