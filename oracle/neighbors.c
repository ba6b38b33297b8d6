/*
 * ORACLE -- test infrastructure only. Nothing in the product path links,
 * loads or calls this file; tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it to check results.
 *
 * CPU restatement of the reference's radius-graph decision
 * (src/mlff_distiller/models/student_model.py:63-109, radius_graph_native):
 *
 *   diff[i,j] = pos[j] - pos[i]                      (float32, :90)
 *   dist[i,j] = torch.norm(diff, dim=2)              (float32, :91)
 *   edge (src=i, dst=j) iff same batch, i != j, dist <= r   (:94-103)
 *   output ordered src-major, then dst (torch.where, :106)
 *
 * torch.norm of a float32 3-vector on the CPU equals, bit for bit,
 * sqrtf(fmaf(z, z, fmaf(y, y, x * x))) with x*x rounded on its own; the
 * test suite re-checks that against torch.norm.  This file is compiled with
 * -ffp-contract=off so no other product is fused.
 *
 * Periodic cells have no counterpart in the reference (its radius graph
 * ignores cell/pbc, student_model.py:694-703).  For orthorhombic cells this
 * oracle defines the minimum-image edge vector per periodic axis as
 *   k  = rintf(dx * (1/L));   dx' = fmaf(-k, L, dx)
 * which is exactly antisymmetric (dx'_ji == -dx'_ij), so d_ij == d_ji.
 * Periodic boxes must have L >= 2*cutoff on every axis, so at most one image
 * of a pair is within the cutoff.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

float oracle_pair_distance(float dx, float dy, float dz)
{
    float xx = dx * dx;
    return sqrtf(fmaf(dz, dz, fmaf(dy, dy, xx)));
}

static inline float min_image(float dx, float L, float invL, int32_t *k_out)
{
    float k = rintf(dx * invL);
    *k_out = (int32_t)k;
    return fmaf(-k, L, dx);
}

static int cmp_i64(const void *a, const void *b)
{
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/*
 * Fill src/dst (and, for periodic molecules, the integer image count k
 * such that  r_e = pos[src] - pos[dst] + k*L  is the minimum image of the
 * reference's edge vector pos[src]-pos[dst]; k is 0 for non-periodic) for
 * all molecules.  Molecule m owns atoms [mol_ptr[m], mol_ptr[m+1]).
 * box[3*m + a] is the orthorhombic edge length on axis a (ignored when
 * pbc[m] == 0).  Returns the number of edges found; if it exceeds cap the
 * arrays hold the first cap edges only (call again with a larger cap).
 * Returns -1 for an invalid periodic box.
 */
int64_t oracle_radius_graph(const float *pos, int64_t n_atoms,
                            const int64_t *mol_ptr, int64_t n_mol,
                            const float *box, const uint8_t *pbc,
                            float cutoff,
                            int64_t *src, int64_t *dst, int32_t *shift,
                            int64_t cap)
{
    (void)n_atoms;
    int64_t e = 0;
    int64_t *nbr = NULL;
    int32_t *nbr_shift = NULL;
    int64_t nbr_cap = 0;
    for (int64_t m = 0; m < n_mol; ++m) {
        int64_t a0 = mol_ptr[m], a1 = mol_ptr[m + 1];
        int periodic = pbc ? pbc[m] != 0 : 0;
        float L[3] = {0, 0, 0}, invL[3] = {0, 0, 0};
        if (periodic) {
            for (int a = 0; a < 3; ++a) {
                L[a] = box[3 * m + a];
                if (!(L[a] >= 2.0f * cutoff)) { free(nbr); free(nbr_shift); return -1; }
                invL[a] = 1.0f / L[a];
            }
        }
        int64_t n = a1 - a0;
        if (n > nbr_cap) {
            nbr_cap = n;
            nbr = (int64_t *)realloc(nbr, sizeof(int64_t) * (size_t)nbr_cap);
            nbr_shift = (int32_t *)realloc(nbr_shift, sizeof(int32_t) * 3 * (size_t)nbr_cap);
        }
        for (int64_t i = a0; i < a1; ++i) {
            int64_t cnt = 0;
            for (int64_t j = a0; j < a1; ++j) {
                if (j == i) continue;
                float dx = pos[3 * j + 0] - pos[3 * i + 0];
                float dy = pos[3 * j + 1] - pos[3 * i + 1];
                float dz = pos[3 * j + 2] - pos[3 * i + 2];
                int32_t kx = 0, ky = 0, kz = 0;
                if (periodic) {
                    dx = min_image(dx, L[0], invL[0], &kx);
                    dy = min_image(dy, L[1], invL[1], &ky);
                    dz = min_image(dz, L[2], invL[2], &kz);
                }
                float d = oracle_pair_distance(dx, dy, dz);
                if (d <= cutoff) {
                    nbr[cnt] = j;
                    /* dx' = (pos[j]-pos[i]) - k*L, so pos[i]-pos[j] + k*L = -dx' */
                    nbr_shift[3 * cnt + 0] = kx;
                    nbr_shift[3 * cnt + 1] = ky;
                    nbr_shift[3 * cnt + 2] = kz;
                    ++cnt;
                }
            }
            /* j loop is ascending, so the row is already sorted by dst */
            for (int64_t c = 0; c < cnt; ++c) {
                if (e < cap) {
                    src[e] = i;
                    dst[e] = nbr[c];
                    if (shift) {
                        shift[3 * e + 0] = nbr_shift[3 * c + 0];
                        shift[3 * e + 1] = nbr_shift[3 * c + 1];
                        shift[3 * e + 2] = nbr_shift[3 * c + 2];
                    }
                }
                ++e;
            }
        }
    }
    free(nbr);
    free(nbr_shift);
    (void)cmp_i64;
    return e;
}

/*
 * Same edge set as oracle_radius_graph for one periodic orthorhombic box,
 * with candidate pairs drawn from a cell grid (cells of edge >= cutoff) so
 * that 1e5-atom boxes finish in seconds.  Every candidate goes through the
 * same float32 decision; rows are sorted by dst afterwards.
 */
int64_t oracle_radius_graph_pbc_cells(const float *pos, int64_t n, const float *box,
                                      float cutoff, int64_t *src, int64_t *dst,
                                      int32_t *shift, int64_t cap)
{
    int nc[3];
    float L[3], invL[3];
    for (int a = 0; a < 3; ++a) {
        L[a] = box[a];
        if (!(L[a] >= 2.0f * cutoff)) return -1;
        invL[a] = 1.0f / L[a];
        nc[a] = (int)floorf(L[a] / (cutoff * 1.0001f)); /* cell edge > cutoff with margin */
        if (nc[a] < 1) nc[a] = 1;
    }
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int64_t *cell_of = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t *head = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncell + 1));
    int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    memset(head, 0, sizeof(int64_t) * (size_t)(ncell + 1));
    for (int64_t i = 0; i < n; ++i) {
        int c[3];
        for (int a = 0; a < 3; ++a) {
            double x = (double)pos[3 * i + a];
            double w = x - (double)L[a] * floor(x / (double)L[a]);
            int ci = (int)floor(w / (double)L[a] * nc[a]);
            if (ci < 0) ci = 0;
            if (ci >= nc[a]) ci = nc[a] - 1;
            c[a] = ci;
        }
        cell_of[i] = ((int64_t)c[0] * nc[1] + c[1]) * nc[2] + c[2];
        head[cell_of[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; ++c) head[c + 1] += head[c];
    {
        int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)ncell);
        memcpy(fill, head, sizeof(int64_t) * (size_t)ncell);
        for (int64_t i = 0; i < n; ++i) order[fill[cell_of[i]]++] = i;
        free(fill);
    }
    int64_t e = 0;
    int64_t buf_cap = 4096;
    int64_t *nb = (int64_t *)malloc(sizeof(int64_t) * (size_t)buf_cap);
    int64_t *nbk = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)buf_cap);
    for (int64_t i = 0; i < n; ++i) {
        int64_t ci = cell_of[i];
        int c0 = (int)(ci / ((int64_t)nc[1] * nc[2]));
        int c1 = (int)((ci / nc[2]) % nc[1]);
        int c2 = (int)(ci % nc[2]);
        int lo[3], hi[3];
        int cc[3] = {c0, c1, c2};
        for (int a = 0; a < 3; ++a) {
            if (nc[a] >= 3) { lo[a] = -1; hi[a] = 1; }
            else { lo[a] = 0; hi[a] = nc[a] - 1; }
        }
        int64_t cnt = 0;
        for (int ox = lo[0]; ox <= hi[0]; ++ox)
        for (int oy = lo[1]; oy <= hi[1]; ++oy)
        for (int oz = lo[2]; oz <= hi[2]; ++oz) {
            int q[3];
            int o[3] = {ox, oy, oz};
            for (int a = 0; a < 3; ++a) {
                if (nc[a] >= 3) q[a] = ((cc[a] + o[a]) % nc[a] + nc[a]) % nc[a];
                else q[a] = o[a];
            }
            int64_t qc = ((int64_t)q[0] * nc[1] + q[1]) * nc[2] + q[2];
            for (int64_t t = head[qc]; t < head[qc + 1]; ++t) {
                int64_t j = order[t];
                if (j == i) continue;
                float dx = pos[3 * j + 0] - pos[3 * i + 0];
                float dy = pos[3 * j + 1] - pos[3 * i + 1];
                float dz = pos[3 * j + 2] - pos[3 * i + 2];
                int32_t k[3];
                dx = min_image(dx, L[0], invL[0], &k[0]);
                dy = min_image(dy, L[1], invL[1], &k[1]);
                dz = min_image(dz, L[2], invL[2], &k[2]);
                if (oracle_pair_distance(dx, dy, dz) <= cutoff) {
                    if (cnt == buf_cap) {
                        buf_cap *= 2;
                        nb = (int64_t *)realloc(nb, sizeof(int64_t) * (size_t)buf_cap);
                        nbk = (int64_t *)realloc(nbk, sizeof(int64_t) * 2 * (size_t)buf_cap);
                    }
                    nb[cnt] = j;
                    /* pack the three small image counts into one key slot */
                    nbk[2 * cnt] = j;
                    nbk[2 * cnt + 1] = ((int64_t)(k[0] + 512) << 20) | ((int64_t)(k[1] + 512) << 10) | (int64_t)(k[2] + 512);
                    ++cnt;
                }
            }
        }
        /* sort (j, packed shift) pairs by j; j values in a row are distinct */
        qsort(nbk, (size_t)cnt, 2 * sizeof(int64_t), cmp_i64);
        for (int64_t c = 0; c < cnt; ++c) {
            if (e < cap) {
                src[e] = i;
                dst[e] = nbk[2 * c];
                if (shift) {
                    int64_t p = nbk[2 * c + 1];
                    shift[3 * e + 0] = (int32_t)((p >> 20) & 1023) - 512;
                    shift[3 * e + 1] = (int32_t)((p >> 10) & 1023) - 512;
                    shift[3 * e + 2] = (int32_t)(p & 1023) - 512;
                }
            }
            ++e;
        }
    }
    free(nb);
    free(nbk);
    free(cell_of);
    free(head);
    free(order);
    return e;
}
