/*
 * btc_oracle.c -- CPU restatement of BTC-GPU's parallel-SGD CP path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke
 * entry and the bench's CPU-baseline leg load it; the product library never
 * links or calls it.  It is written for clarity, not speed, and follows the
 * reference algorithm step by step:
 *
 *   hx bucket code ............. block.cu:38-50
 *   tree routing ............... block.cu:53-88   (search_block / compare)
 *   leaf split ................. block.cu:90-152  (Create_Btree)
 *   incremental blocking ....... block.cu:154-401 (tensor_block)
 *   axis conflict .............. block.cu:413-456 (find_conflict_x / axis_conflict)
 *   conflict-free strata ....... block.cu:926-1148 (compare_tree / tree_conflict /
 *                                search_parallel_block_Tree): greedy lowest-id
 *                                maximal sets; the tree BFS of the reference
 *                                removes exactly the blocks that conflict on some
 *                                axis, so a pairwise test is used here
 *   GPU target ................. block.cu:567-619
 *   balancing + padding ........ block.cu:524-565, 660-697
 *   coe weights ................ block.cu:470-513 (union-find per axis)
 *   flattening ................. block.cu:1151-1190 (Preproccess_list)
 *   SGD update rule ............ sgd_Kernel.cu:336-351 (pre-update rows, coe*lr)
 *   lock-free variant .......... sgd_Kernel.cu:401-451, block.cu:1192-1217
 *   test metrics ............... sgd_Kernel.cu:85-99, 188-199
 *
 * Build with -ffp-contract=off: the update rule is evaluated exactly as
 * written (coe*lr)*((e*bc)-(reg*a)) with an explicit fma for the dot.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_ALLOC 3
#define ORC_ERR_RANGE 8

/* ---- hx: bucket index of coordinate `num` at `level` (block.cu:38-50) ----
 * n_1 = (end-start+1)/2^(level-1) computed in double and stored as float,
 * n_2 = floor(num / n_1) computed in float.  The reference keeps the low
 * `level` bits of n_2 MSB-first; position 0 is bit level-1. */
static int orc_hx(int end, int level, int num, int64_t *out)
{
    float n1 = (float)((double)(end + 1) / pow(2.0, (double)(level - 1)));
    float q = (float)num / n1;
    float f = floorf(q);
    if (!(f >= 0.0f) || f >= 2147483648.0f)
        return ORC_ERR_RANGE; /* int conversion would overflow in the reference */
    *out = (int64_t)f;
    return ORC_OK;
}

/* bits at positions 1..L-1 of the level-g vector of n2, read MSB first */
static uint64_t orc_prefix(int64_t n2, int g, int L)
{
    if (L <= 1)
        return 0;
    uint64_t v = (uint64_t)n2 >> (g - L);
    return v & ((1ULL << (L - 1)) - 1ULL);
}

typedef struct {
    int h;
    int block;
    int left, right;
    int len[3];
    uint64_t code[3]; /* positions 1..len-1, MSB first */
} orc_node;

typedef struct {
    int level[3];
    uint64_t code[3];
    int nnz;
    int32_t *ent; /* entry indices, capacity block_s */
} orc_block;

typedef struct orc_sched {
    int I, J, K, block_s, pss, resident;
    int nblocks;
    orc_block *blocks;
    int nnodes, cap_nodes;
    orc_node *nodes;
    /* conflict-free strata (before balancing) */
    int nstrata;
    int *strata_off; /* nstrata+1 */
    int *strata_ids;
    int max_parallel_cf;
    int target;
    /* balanced groups = GPU schedule */
    int ngroups;
    int *group_off; /* ngroups+1 */
    int *slot_ids;
    double *slot_coe; /* 3 per slot */
    int max_parallel;
    /* branch counters for fixtures */
    int64_t n_split, n_flag0, n_dup, n_empty_resplit;
    int gmax[3];
} orc_sched;

static int axis_of_h(int h)
{
    int t = h % 3;
    return t == 1 ? 0 : (t == 2 ? 1 : 2);
}

static int new_node(orc_sched *s)
{
    if (s->nnodes == s->cap_nodes) {
        int nc = s->cap_nodes ? s->cap_nodes * 2 : 1024;
        orc_node *nn = (orc_node *)realloc(s->nodes, (size_t)nc * sizeof(orc_node));
        if (!nn)
            return -1;
        s->nodes = nn;
        s->cap_nodes = nc;
    }
    return s->nnodes++;
}

/* Create_Btree (block.cu:90-152): left child keeps old_id, right gets new_id;
 * the split axis follows the node's depth h. */
static int create_btree(orc_sched *s, int node, int old_id, int new_id)
{
    int l = new_node(s), r = new_node(s);
    if (l < 0 || r < 0)
        return ORC_ERR_ALLOC;
    orc_node *p = &s->nodes[node];
    int a = axis_of_h(p->h);
    p->block = -1;
    orc_node *L = &s->nodes[l], *R = &s->nodes[r];
    *L = *p;
    *R = *p;
    L->h = R->h = p->h + 1;
    L->left = L->right = R->left = R->right = -1;
    L->len[a] = R->len[a] = p->len[a] + 1;
    L->code[a] = p->code[a] << 1;
    R->code[a] = (p->code[a] << 1) | 1ULL;
    L->block = old_id;
    R->block = new_id;
    p->left = l;
    p->right = r;
    return ORC_OK;
}

static int coord(const int32_t *xyz, int e, int a) { return xyz[3 * (int64_t)e + a]; }

/* tensor_block (block.cu:154-401). */
static int orc_blocking(orc_sched *s, const int32_t *xyz, int64_t n)
{
    int bs = s->block_s;
    int end[3] = {s->I, s->J, s->K};
    int g[3] = {1, 1, 1};
    /* the reference sizes its block array by train_nnz (block.cu:1256); more
     * blocks than entries overruns it there, so such inputs have no reference
     * answer.  The oracle grows its array and reports the count. */
    int64_t cap_blocks = n > 0 ? n : 1;
    if (cap_blocks > (1 << 30))
        return ORC_ERR_ARG;
    s->blocks = (orc_block *)calloc((size_t)cap_blocks + 1, sizeof(orc_block));
    if (!s->blocks)
        return ORC_ERR_ALLOC;
    int root = new_node(s);
    if (root < 0)
        return ORC_ERR_ALLOC;
    orc_node *rt = &s->nodes[root];
    memset(rt, 0, sizeof(*rt));
    rt->h = 1;
    rt->block = 0;
    rt->left = rt->right = -1;
    for (int a = 0; a < 3; a++)
        rt->len[a] = 1;
    orc_block *b0 = &s->blocks[0];
    b0->level[0] = b0->level[1] = b0->level[2] = 1;
    b0->ent = (int32_t *)malloc((size_t)bs * sizeof(int32_t));
    if (!b0->ent)
        return ORC_ERR_ALLOC;
    int nb = 1;
    int32_t *t1 = (int32_t *)malloc((size_t)bs * sizeof(int32_t));
    int32_t *t2 = (int32_t *)malloc((size_t)bs * sizeof(int32_t));
    if (!t1 || !t2)
        return ORC_ERR_ALLOC;

    for (int64_t i = 0; i < n; i++) {
        int64_t pc[3];
        for (int a = 0; a < 3; a++)
            if (orc_hx(end[a], g[a], coord(xyz, (int)i, a), &pc[a]))
                return ORC_ERR_RANGE;
        int node = root;
        while (s->nodes[node].left != -1) {
            int a = axis_of_h(s->nodes[node].h);
            orc_node *lc = &s->nodes[s->nodes[node].left];
            int L = lc->len[a];
            if (orc_prefix(pc[a], g[a], L) == lc->code[a])
                node = s->nodes[node].left;
            else
                node = s->nodes[node].right;
        }
        int id = s->nodes[node].block;
        if (s->blocks[id].nnz < bs) {
            s->blocks[id].ent[s->blocks[id].nnz++] = (int32_t)i;
            continue;
        }
        int flag = 0;
        while (flag == 0) {
            orc_block *B = &s->blocks[id];
            int a;
            if (B->level[0] == B->level[1] && B->level[1] == B->level[2])
                a = 0;
            else if (B->level[1] < B->level[0])
                a = 1;
            else if (B->level[2] < B->level[1])
                a = 2;
            else
                return ORC_ERR_ARG; /* unreachable for round-robin levels */
            B->level[a]++;
            if (B->level[a] > g[a])
                g[a] = B->level[a];
            if (g[a] > 63)
                return ORC_ERR_RANGE;
            int rc = create_btree(s, node, id, nb);
            if (rc)
                return rc;
            if (nb >= cap_blocks) {
                orc_block *grown = (orc_block *)realloc(s->blocks, (size_t)(2 * cap_blocks + 1) * sizeof(orc_block));
                if (!grown)
                    return ORC_ERR_ALLOC;
                memset(grown + cap_blocks + 1, 0, (size_t)cap_blocks * sizeof(orc_block));
                s->blocks = grown;
                cap_blocks *= 2;
            }
            B = &s->blocks[id];
            orc_block *NB = &s->blocks[nb];
            NB->nnz = 0;
            NB->level[0] = B->level[0];
            NB->level[1] = B->level[1];
            NB->level[2] = B->level[2];
            NB->code[0] = B->code[0];
            NB->code[1] = B->code[1];
            NB->code[2] = B->code[2];
            NB->code[a] = (B->code[a] << 1) | 1ULL;
            B->code[a] = B->code[a] << 1;
            NB->ent = (int32_t *)malloc((size_t)bs * sizeof(int32_t));
            if (!NB->ent)
                return ORC_ERR_ALLOC;
            s->n_split++;
            int n1 = 0, n2 = 0;
            for (int j = 0; j < B->nnz; j++) {
                int64_t hv;
                if (orc_hx(end[a], g[a], coord(xyz, B->ent[j], a), &hv))
                    return ORC_ERR_RANGE;
                if ((hv & 1) == 0)
                    t1[n1++] = B->ent[j];
                else
                    t2[n2++] = B->ent[j];
            }
            int64_t hp;
            if (orc_hx(end[a], g[a], coord(xyz, (int)i, a), &hp))
                return ORC_ERR_RANGE;
            int bit = (int)(hp & 1);
            if (n1 < bs && n2 < bs) {
                flag = 1;
                if (bit == 0)
                    t1[n1++] = (int32_t)i;
                else
                    t2[n2++] = (int32_t)i;
                memcpy(B->ent, t1, (size_t)n1 * sizeof(int32_t));
                B->nnz = n1;
                memcpy(NB->ent, t2, (size_t)n2 * sizeof(int32_t));
                NB->nnz = n2;
            } else {
                s->n_flag0++;
                if (bit == 0) {
                    /* id stays: old <- t1, new <- t2 */
                    memcpy(B->ent, t1, (size_t)n1 * sizeof(int32_t));
                    B->nnz = n1;
                    memcpy(NB->ent, t2, (size_t)n2 * sizeof(int32_t));
                    NB->nnz = n2;
                    node = s->nodes[node].left;
                    if (n1 == 0)
                        s->n_empty_resplit++;
                } else {
                    /* id moves to the new block; the reference stores t1 and then
                     * t2 into that same block, so the old block keeps its previous
                     * entries (block.cu:244-253) */
                    memcpy(NB->ent, t2, (size_t)n2 * sizeof(int32_t));
                    NB->nnz = n2;
                    if (n2 > 0)
                        s->n_dup++;
                    else
                        s->n_empty_resplit++;
                    id = nb;
                    node = s->nodes[node].right;
                }
            }
            nb++;
        }
    }
    free(t1);
    free(t2);
    s->nblocks = nb;
    s->gmax[0] = g[0];
    s->gmax[1] = g[1];
    s->gmax[2] = g[2];
    return ORC_OK;
}

/* find_conflict_x (block.cu:413-430): 1 if the two ids agree on positions
 * 1..min(level)-1 (always when the shorter level is 1). */
static int axis_conflict(const orc_sched *s, int a_id, int b_id, int a)
{
    const orc_block *A = &s->blocks[a_id], *B = &s->blocks[b_id];
    int la = A->level[a], lb = B->level[a];
    int L = la < lb ? la : lb;
    if (L == 1)
        return 1;
    uint64_t pa = A->code[a] >> (la - L);
    uint64_t pb = B->code[a] >> (lb - L);
    return pa == pb;
}

static int any_conflict(const orc_sched *s, int a_id, int b_id)
{
    return axis_conflict(s, a_id, b_id, 0) || axis_conflict(s, a_id, b_id, 1) ||
           axis_conflict(s, a_id, b_id, 2);
}

/* search_parallel_block_Tree (block.cu:1024-1148) */
static int orc_strata(orc_sched *s)
{
    int nb = s->nblocks;
    int *rem = (int *)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
    int *chosen = (int *)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
    s->strata_ids = (int *)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
    s->strata_off = (int *)malloc((size_t)(nb + 2) * sizeof(int));
    if (!rem || !chosen || !s->strata_ids || !s->strata_off)
        return ORC_ERR_ALLOC;
    int nrem = 0;
    for (int i = 0; i < nb; i++)
        if (s->blocks[i].nnz != 0)
            rem[nrem++] = i;
    int ns = 0, pos = 0, maxp = 0;
    s->strata_off[0] = 0;
    while (nrem > 0) {
        int nch = 0, keep = 0;
        for (int k = 0; k < nrem; k++) {
            int c = rem[k];
            int ok = 1;
            for (int m = 0; m < nch && ok; m++)
                if (any_conflict(s, chosen[m], c))
                    ok = 0;
            if (ok)
                chosen[nch++] = c;
            else
                rem[keep++] = c;
        }
        nrem = keep;
        for (int m = 0; m < nch; m++)
            s->strata_ids[pos++] = chosen[m];
        ns++;
        s->strata_off[ns] = pos;
        if (nch > maxp)
            maxp = nch;
    }
    s->nstrata = ns;
    s->max_parallel_cf = maxp;
    free(rem);
    free(chosen);
    return ORC_OK;
}

/* configured_gpu_block_target / gpu_block_target (block.cu:577-619).
 * `resident` stands for SMs x maxBlocksPerSM; 0 means no device. */
static int orc_target(int max_parallel, int block_num, int pss, int resident)
{
    int target;
    if (pss > 0) {
        target = pss;
    } else {
        target = max_parallel > 0 ? max_parallel : 1;
        if (resident > 0 && resident < target)
            target = resident;
        if (target < 1)
            target = 1;
        if (block_num > 0 && target > block_num)
            target = block_num;
    }
    if (target < 1)
        target = 1;
    if (block_num > 0 && target > block_num)
        target = block_num;
    return target;
}

/* select_min_conflict_block (block.cu:524-565) */
static int select_min_conflict(const orc_sched *s, const int *seq, int nseq)
{
    int best = -1, best_score = 0, best_work = 0;
    for (int i = 0; i < s->nblocks; i++) {
        if (s->blocks[i].nnz == 0)
            continue;
        int in = 0;
        for (int k = 0; k < nseq; k++)
            if (seq[k] == i) {
                in = 1;
                break;
            }
        if (in)
            continue;
        int score = 0;
        for (int k = 0; k < nseq; k++)
            for (int a = 0; a < 3; a++)
                score += axis_conflict(s, seq[k], i, a);
        int work = s->blocks[i].nnz;
        if (best == -1 || score < best_score || (score == best_score && work < best_work)) {
            best = i;
            best_score = score;
            best_work = work;
        }
    }
    return best;
}

static int uf_find(int *p, int i)
{
    while (p[i] != i) {
        p[i] = p[p[i]];
        i = p[i];
    }
    return i;
}

/* update_conflict_weights (block.cu:470-513) */
static void coe_weights(const orc_sched *s, const int *ids, int n, double *coe /* 3*n */)
{
    int *par = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    long long *sum = (long long *)malloc((size_t)(n > 0 ? n : 1) * sizeof(long long));
    for (int a = 0; a < 3; a++) {
        for (int i = 0; i < n; i++) {
            par[i] = i;
            sum[i] = 0;
        }
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++)
                if (axis_conflict(s, ids[i], ids[j], a)) {
                    int ra = uf_find(par, i), rb = uf_find(par, j);
                    if (ra != rb)
                        par[rb] = ra;
                }
        for (int i = 0; i < n; i++) {
            int c = s->blocks[ids[i]].nnz > 0 ? s->blocks[ids[i]].nnz : 1;
            sum[uf_find(par, i)] += c;
        }
        for (int i = 0; i < n; i++) {
            int c = s->blocks[ids[i]].nnz > 0 ? s->blocks[ids[i]].nnz : 1;
            long long t = sum[uf_find(par, i)];
            coe[3 * i + a] = t > 0 ? (double)c / (double)(int)t : 1.0;
        }
    }
    free(par);
    free(sum);
}

/* balance_parallel_sequences_for_gpu (block.cu:660-697) + Preproccess_list
 * (block.cu:1151-1190) */
static int orc_balance(orc_sched *s)
{
    int target = s->target;
    int total = s->strata_off[s->nstrata];
    /* upper bound on groups: one per stratum chunk */
    int maxg = total + s->nstrata + 1;
    s->group_off = (int *)malloc((size_t)(maxg + 1) * sizeof(int));
    int cap_slots = maxg * target + 1;
    s->slot_ids = (int *)malloc((size_t)cap_slots * sizeof(int));
    s->slot_coe = (double *)malloc((size_t)cap_slots * 3 * sizeof(double));
    if (!s->group_off || !s->slot_ids || !s->slot_coe)
        return ORC_ERR_ALLOC;
    int ng = 0, pos = 0;
    s->group_off[0] = 0;
    for (int st = 0; st < s->nstrata; st++) {
        int cur = 0;
        for (int k = s->strata_off[st]; k < s->strata_off[st + 1]; k++) {
            int id = s->strata_ids[k];
            if (s->blocks[id].nnz == 0)
                continue;
            s->slot_ids[pos++] = id;
            cur++;
            if (cur == target) {
                ng++;
                s->group_off[ng] = pos;
                cur = 0;
            }
        }
        if (cur > 0) {
            ng++;
            s->group_off[ng] = pos;
        }
    }
    /* pad each group; groups only grow at their tail, so rebuild into a new array */
    int *ids2 = (int *)malloc((size_t)(ng * target + 1) * sizeof(int));
    int *off2 = (int *)malloc((size_t)(ng + 1) * sizeof(int));
    if (!ids2 || !off2)
        return ORC_ERR_ALLOC;
    int p2 = 0, maxp = 0;
    off2[0] = 0;
    for (int gi = 0; gi < ng; gi++) {
        int start = p2;
        for (int k = s->group_off[gi]; k < s->group_off[gi + 1]; k++)
            ids2[p2++] = s->slot_ids[k];
        while (p2 - start < target) {
            int b = select_min_conflict(s, ids2 + start, p2 - start);
            if (b == -1)
                break;
            ids2[p2++] = b;
        }
        off2[gi + 1] = p2;
        if (p2 - start > maxp)
            maxp = p2 - start;
    }
    free(s->slot_ids);
    free(s->group_off);
    s->slot_ids = ids2;
    s->group_off = off2;
    s->ngroups = ng;
    s->max_parallel = maxp;
    free(s->slot_coe);
    s->slot_coe = (double *)malloc((size_t)(p2 + 1) * 3 * sizeof(double));
    if (!s->slot_coe)
        return ORC_ERR_ALLOC;
    for (int gi = 0; gi < ng; gi++)
        coe_weights(s, s->slot_ids + off2[gi], off2[gi + 1] - off2[gi], s->slot_coe + 3 * (size_t)off2[gi]);
    return ORC_OK;
}

void orc_free(orc_sched *s)
{
    if (!s)
        return;
    if (s->blocks) {
        for (int i = 0; i < s->nblocks + 1; i++)
            free(s->blocks[i].ent);
        free(s->blocks);
    }
    free(s->nodes);
    free(s->strata_off);
    free(s->strata_ids);
    free(s->group_off);
    free(s->slot_ids);
    free(s->slot_coe);
    free(s);
}

/* Build the whole schedule from entries already in the reference's
 * (shuffled) order.  xyz is n x 3, 0-based. */
int orc_build(const int32_t *xyz, int64_t n, int I, int J, int K, int block_s, int pss,
              int resident, orc_sched **out)
{
    *out = NULL;
    if (n < 0 || n > 0x7fffffff || block_s <= 0 || I <= 0 || J <= 0 || K <= 0 || pss < 0)
        return ORC_ERR_ARG;
    orc_sched *s = (orc_sched *)calloc(1, sizeof(orc_sched));
    if (!s)
        return ORC_ERR_ALLOC;
    s->I = I;
    s->J = J;
    s->K = K;
    s->block_s = block_s;
    s->pss = pss;
    s->resident = resident;
    int rc = orc_blocking(s, xyz, n);
    if (!rc)
        rc = orc_strata(s);
    if (!rc) {
        s->target = orc_target(s->max_parallel_cf, s->nblocks, pss, resident);
        rc = orc_balance(s);
    }
    if (rc) {
        orc_free(s);
        return rc;
    }
    *out = s;
    return ORC_OK;
}

/* ---- queries ---- */
int orc_num_blocks(const orc_sched *s) { return s->nblocks; }
int orc_num_strata(const orc_sched *s) { return s->nstrata; }
int orc_num_groups(const orc_sched *s) { return s->ngroups; }
int orc_num_slots(const orc_sched *s) { return s->group_off[s->ngroups]; }

/* info[8] = nblocks, nstrata, max_parallel_cf, target, ngroups, nslots, max_parallel, 0
 * cnt[4] = splits, flag0 re-splits, duplicating re-splits, empty re-splits
 * gmax[3] = final global levels */
void orc_info(const orc_sched *s, int32_t *info, int64_t *cnt, int32_t *gmax)
{
    info[0] = s->nblocks;
    info[1] = s->nstrata;
    info[2] = s->max_parallel_cf;
    info[3] = s->target;
    info[4] = s->ngroups;
    info[5] = s->group_off[s->ngroups];
    info[6] = s->max_parallel;
    info[7] = 0;
    cnt[0] = s->n_split;
    cnt[1] = s->n_flag0;
    cnt[2] = s->n_dup;
    cnt[3] = s->n_empty_resplit;
    gmax[0] = s->gmax[0];
    gmax[1] = s->gmax[1];
    gmax[2] = s->gmax[2];
}

/* per block: nnz, level_x, level_y, level_z; codes as 3 uint64 */
void orc_blocks(const orc_sched *s, int32_t *meta /* 4*nb */, uint64_t *codes /* 3*nb */)
{
    for (int i = 0; i < s->nblocks; i++) {
        meta[4 * i] = s->blocks[i].nnz;
        for (int a = 0; a < 3; a++) {
            meta[4 * i + 1 + a] = s->blocks[i].level[a];
            codes[3 * i + a] = s->blocks[i].code[a];
        }
    }
}

int orc_block_entries(const orc_sched *s, int b, int32_t *out)
{
    memcpy(out, s->blocks[b].ent, (size_t)s->blocks[b].nnz * sizeof(int32_t));
    return s->blocks[b].nnz;
}

void orc_strata_arrays(const orc_sched *s, int32_t *off /* nstrata+1 */, int32_t *ids)
{
    for (int i = 0; i <= s->nstrata; i++)
        off[i] = s->strata_off[i];
    for (int i = 0; i < s->strata_off[s->nstrata]; i++)
        ids[i] = s->strata_ids[i];
}

void orc_groups(const orc_sched *s, int32_t *off /* ngroups+1 */, int32_t *ids, double *coe)
{
    int ns = s->group_off[s->ngroups];
    for (int i = 0; i <= s->ngroups; i++)
        off[i] = s->group_off[i];
    for (int i = 0; i < ns; i++) {
        ids[i] = s->slot_ids[i];
        coe[3 * i] = s->slot_coe[3 * i];
        coe[3 * i + 1] = s->slot_coe[3 * i + 1];
        coe[3 * i + 2] = s->slot_coe[3 * i + 2];
    }
}

/* ---- SGD: serial FP64 replay of the GPUs kernel rule (sgd_Kernel.cu:336-351)
 * over strata -> slots -> entries in block order.  Factors row-major [n][R].
 * Returns the number of executed updates. */
int64_t orc_sgd_epoch(const orc_sched *s, const int32_t *xyz, const double *val, int R,
                      double lr, double reg, double *A, double *B, double *C)
{
    int64_t upd = 0;
    double *av = (double *)malloc((size_t)R * 3 * sizeof(double));
    double *bv = av + R, *cv = av + 2 * R;
    int ns = s->group_off[s->ngroups];
    for (int k = 0; k < ns; k++) {
        const orc_block *blk = &s->blocks[s->slot_ids[k]];
        double cx = s->slot_coe[3 * k] * lr;
        double cy = s->slot_coe[3 * k + 1] * lr;
        double cz = s->slot_coe[3 * k + 2] * lr;
        for (int t = 0; t < blk->nnz; t++) {
            int e = blk->ent[t];
            double *Ar = A + (size_t)xyz[3 * (int64_t)e] * R;
            double *Br = B + (size_t)xyz[3 * (int64_t)e + 1] * R;
            double *Cr = C + (size_t)xyz[3 * (int64_t)e + 2] * R;
            double dot = 0.0;
            for (int q = 0; q < R; q++) {
                av[q] = Ar[q];
                bv[q] = Br[q];
                cv[q] = Cr[q];
                dot = fma(av[q], bv[q] * cv[q], dot);
            }
            double err = val[e] - dot;
            for (int q = 0; q < R; q++) {
                double bc = bv[q] * cv[q];
                double ac = av[q] * cv[q];
                double ab = av[q] * bv[q];
                Ar[q] = Ar[q] + cx * (err * bc - reg * av[q]);
                Br[q] = Br[q] + cy * (err * ac - reg * bv[q]);
                Cr[q] = Cr[q] + cz * (err * ab - reg * cv[q]);
            }
            upd++;
        }
    }
    free(av);
    return upd;
}

/* The lock-free variant (tensor_LF, sgd_Kernel.cu:401-451; its entry list
 * ToMatrix_LF, block.cu:1192-1217): the conflict-free strata in order, every
 * block of a stratum in order, every entry of a block in order, no coe
 * weights.  The rows are updated in place element by element: A first, B
 * from the new A, C from the new A and B.  Rounding as written in this
 * restatement (the reference's own contraction is the compiler's choice):
 * dot = fma(a * b, c, dot), x' = x + lr * ((e * u) * v - reg * x).  The
 * reference reads one stratum count past the strata it fills (num_LF has
 * num_parallel entries for num_parallel - 1 strata); only the filled strata
 * are replayed here. */
int64_t orc_lf_epoch(const orc_sched *s, const int32_t *xyz, const double *val, int R, double lr, double reg,
                     double *A, double *B, double *C)
{
    int64_t upd = 0;
    for (int i = 0; i < s->nstrata; i++)
        for (int m = s->strata_off[i]; m < s->strata_off[i + 1]; m++) {
            const orc_block *blk = &s->blocks[s->strata_ids[m]];
            for (int t = 0; t < blk->nnz; t++) {
                int e = blk->ent[t];
                double *Ar = A + (size_t)xyz[3 * (int64_t)e] * R;
                double *Br = B + (size_t)xyz[3 * (int64_t)e + 1] * R;
                double *Cr = C + (size_t)xyz[3 * (int64_t)e + 2] * R;
                double dot = 0.0;
                for (int q = 0; q < R; q++)
                    dot = fma(Ar[q] * Br[q], Cr[q], dot);
                double err = val[e] - dot;
                for (int q = 0; q < R; q++) {
                    Ar[q] = Ar[q] + lr * ((err * Br[q]) * Cr[q] - reg * Ar[q]);
                    Br[q] = Br[q] + lr * ((err * Ar[q]) * Cr[q] - reg * Br[q]);
                    Cr[q] = Cr[q] + lr * ((err * Br[q]) * Ar[q] - reg * Cr[q]);
                }
                upd++;
            }
        }
    return upd;
}

/* compute_metrics_gpu restated (sgd_Kernel.cu:85-99, 188-199):
 * out[0]=SSE out[1]=SAE out[2]=sum ref^2; rmse = sqrt(SSE/n) etc. */
void orc_metrics(const int32_t *xyz, const double *val, int64_t n, int R, const double *A,
                 const double *B, const double *C, double *out)
{
    double sse = 0, sae = 0, r2 = 0;
    for (int64_t i = 0; i < n; i++) {
        const double *Ar = A + (size_t)xyz[3 * i] * R;
        const double *Br = B + (size_t)xyz[3 * i + 1] * R;
        const double *Cr = C + (size_t)xyz[3 * i + 2] * R;
        double dot = 0.0;
        for (int q = 0; q < R; q++)
            dot = fma(Ar[q], Br[q] * Cr[q], dot);
        double err = val[i] - dot;
        sae += fabs(err);
        sse += err * err;
        r2 += val[i] * val[i];
    }
    out[0] = sse;
    out[1] = sae;
    out[2] = r2;
}

/* Expose hx for the tests of the float-rounding quirk. */
int orc_hx_public(int end, int level, int num, int64_t *out) { return orc_hx(end, level, num, out); }

/* ---- replay over a flattened schedule ----------------------------------
 * slot k covers entry indices ent[soff[k] .. soff[k+1]) of xyz/val and has
 * weights coe[3k..3k+2]; slots [s0, s1) are replayed in order.  This is the
 * serial CPU baseline of the reference update rule (sgd_Kernel.cu:336-351). */
int64_t orc_sgd_replay(int64_t s0, int64_t s1, const int64_t *soff, const int32_t *ent,
                       const double *coe, const int32_t *xyz, const double *val, int R, double lr,
                       double reg, double *A, double *B, double *C)
{
    int64_t upd = 0;
    double av[256], bv[256], cv[256];
    if (R > 256)
        return -1;
    for (int64_t k = s0; k < s1; k++) {
        double cx = coe[3 * k] * lr, cy = coe[3 * k + 1] * lr, cz = coe[3 * k + 2] * lr;
        for (int64_t t = soff[k]; t < soff[k + 1]; t++) {
            int e = ent[t];
            double *Ar = A + (size_t)xyz[3 * (int64_t)e] * R;
            double *Br = B + (size_t)xyz[3 * (int64_t)e + 1] * R;
            double *Cr = C + (size_t)xyz[3 * (int64_t)e + 2] * R;
            double dot = 0.0;
            for (int q = 0; q < R; q++) {
                av[q] = Ar[q];
                bv[q] = Br[q];
                cv[q] = Cr[q];
                dot = fma(av[q], bv[q] * cv[q], dot);
            }
            double err = val[e] - dot;
            for (int q = 0; q < R; q++) {
                Ar[q] = Ar[q] + cx * (err * (bv[q] * cv[q]) - reg * av[q]);
                Br[q] = Br[q] + cy * (err * (av[q] * cv[q]) - reg * bv[q]);
                Cr[q] = Cr[q] + cz * (err * (av[q] * bv[q]) - reg * cv[q]);
            }
            upd++;
        }
    }
    return upd;
}

/* Multi-threaded replay: the entries of one group (stratum) are split
 * across threads that read rows and add deltas with atomic compare-and-swap,
 * the reference GPU kernel's Hogwild model on host cores; a barrier separates
 * groups.  Groups [g0, g1) of goff[] (slot offsets per group). */
#include <pthread.h>

typedef struct {
    int tid, nthreads;
    int64_t g0, g1;
    const int64_t *goff, *soff;
    const int32_t *ent;
    const double *coe;
    const int32_t *xyz;
    const double *val;
    int R;
    double lr, reg;
    double *A, *B, *C;
    pthread_barrier_t *bar;
    int64_t upd;
} orc_mt_arg;

static double ld_relaxed(const double *p)
{
    uint64_t u = __atomic_load_n((const uint64_t *)p, __ATOMIC_RELAXED);
    double d;
    memcpy(&d, &u, 8);
    return d;
}

static void add_atomic(double *p, double v)
{
    uint64_t *u = (uint64_t *)p;
    uint64_t old = __atomic_load_n(u, __ATOMIC_RELAXED), nw;
    do {
        double d;
        memcpy(&d, &old, 8);
        d = d + v;
        memcpy(&nw, &d, 8);
    } while (!__atomic_compare_exchange_n(u, &old, nw, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
}

static void *orc_mt_worker(void *vp)
{
    orc_mt_arg *a = (orc_mt_arg *)vp;
    double av[256], bv[256], cv[256];
    int R = a->R;
    for (int64_t g = a->g0; g < a->g1; g++) {
        int64_t s0 = a->goff[g], s1 = a->goff[g + 1];
        int64_t e0 = a->soff[s0], e1 = a->soff[s1];
        int64_t n = e1 - e0;
        int64_t lo = e0 + n * a->tid / a->nthreads, hi = e0 + n * (a->tid + 1) / a->nthreads;
        int64_t k = s0;
        for (int64_t t = lo; t < hi; t++) {
            while (a->soff[k + 1] <= t)
                k++;
            double cx = a->coe[3 * k] * a->lr, cy = a->coe[3 * k + 1] * a->lr, cz = a->coe[3 * k + 2] * a->lr;
            int e = a->ent[t];
            double *Ar = a->A + (size_t)a->xyz[3 * (int64_t)e] * R;
            double *Br = a->B + (size_t)a->xyz[3 * (int64_t)e + 1] * R;
            double *Cr = a->C + (size_t)a->xyz[3 * (int64_t)e + 2] * R;
            double dot = 0.0;
            for (int q = 0; q < R; q++) {
                av[q] = ld_relaxed(Ar + q);
                bv[q] = ld_relaxed(Br + q);
                cv[q] = ld_relaxed(Cr + q);
                dot = fma(av[q], bv[q] * cv[q], dot);
            }
            double err = a->val[e] - dot;
            for (int q = 0; q < R; q++) {
                add_atomic(Ar + q, cx * (err * (bv[q] * cv[q]) - a->reg * av[q]));
                add_atomic(Br + q, cy * (err * (av[q] * cv[q]) - a->reg * bv[q]));
                add_atomic(Cr + q, cz * (err * (av[q] * bv[q]) - a->reg * cv[q]));
            }
            a->upd++;
        }
        pthread_barrier_wait(a->bar);
    }
    return NULL;
}

int64_t orc_sgd_replay_mt(int64_t g0, int64_t g1, const int64_t *goff, const int64_t *soff,
                          const int32_t *ent, const double *coe, const int32_t *xyz, const double *val,
                          int R, double lr, double reg, double *A, double *B, double *C, int threads)
{
    if (threads < 1 || threads > 512 || R > 256)
        return -1;
    pthread_t th[512];
    orc_mt_arg args[512];
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)threads);
    for (int t = 0; t < threads; t++) {
        orc_mt_arg *a = &args[t];
        a->tid = t;
        a->nthreads = threads;
        a->g0 = g0;
        a->g1 = g1;
        a->goff = goff;
        a->soff = soff;
        a->ent = ent;
        a->coe = coe;
        a->xyz = xyz;
        a->val = val;
        a->R = R;
        a->lr = lr;
        a->reg = reg;
        a->A = A;
        a->B = B;
        a->C = C;
        a->bar = &bar;
        a->upd = 0;
    }
    for (int t = 1; t < threads; t++)
        pthread_create(&th[t], NULL, orc_mt_worker, &args[t]);
    orc_mt_worker(&args[0]);
    int64_t upd = args[0].upd;
    for (int t = 1; t < threads; t++) {
        pthread_join(th[t], NULL);
        upd += args[t].upd;
    }
    pthread_barrier_destroy(&bar);
    return upd;
}
