/*
 * ORACLE — test infrastructure only.  A float64 CPU restatement of the
 * reference's self-gravity hot path (Khaserdene/real-astronomy-simulation),
 * that the tests compare the GPU engine against, and the timed CPU baseline.
 * Nothing in the shipped package links or calls this file.
 *
 * Pinned against golden fixtures produced by running the reference's own
 * Python source (tests/golden/gen_golden.py; tests/test_oracle_golden.py).
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (oracle/oracle.py).
 * -ffp-contract=off keeps every multiply and add separately rounded, matching
 * the reference's float64 expression order.
 *
 * Layouts: positions / velocities / accelerations are (n, 3) row-major
 * float64, masses (n,) float64, node arrays indexed like the reference
 * (leaves 0..n-1, internal nodes n..2n-2, root = n).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ direct
 * core/solvers/gravity.py:13-26 compute_acc_direct: for every i, loop over
 * ALL j (the i == j term adds exactly zero), d = x_j - x_i,
 * r2 = d.d + eps2, inv = 1/sqrt(r2), a += (G*m_j*inv*inv*inv) * d. */
static void direct_one(const double *pos, const double *mass, int64_t n,
                       double G, double eps2, int64_t i, double *out) {
    const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int64_t j = 0; j < n; ++j) {
        const double dx = pos[3 * j] - px;
        const double dy = pos[3 * j + 1] - py;
        const double dz = pos[3 * j + 2] - pz;
        const double r2 = dx * dx + dy * dy + dz * dz + eps2;
        const double inv = 1.0 / sqrt(r2);
        const double s = G * mass[j] * inv * inv * inv;
        ax += s * dx;
        ay += s * dy;
        az += s * dz;
    }
    out[0] = ax;
    out[1] = ay;
    out[2] = az;
}

void orc_direct_acc(const double *pos, const double *mass, double *acc,
                    int64_t n, double G, double eps2) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) direct_one(pos, mass, n, G, eps2, i, acc + 3 * i);
}

/* Same sum for a subset of targets (sampled-target FP64 checks). */
void orc_direct_acc_targets(const double *pos, const double *mass, int64_t n,
                            const int64_t *targets, int64_t nt, double G,
                            double eps2, double *acc) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < nt; ++t)
        direct_one(pos, mass, n, G, eps2, targets[t], acc + 3 * t);
}

/* Per-target potential sum_{j != i} m_j / sqrt(r2): the inner loop of
 * core/solvers/gravity.py:49-55. */
void orc_phi_targets(const double *pos, const double *mass, int64_t n,
                     const int64_t *targets, int64_t nt, double eps2,
                     double *phi) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t i = targets[t];
        const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        double s = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            if (j == i) continue;
            const double dx = pos[3 * j] - px;
            const double dy = pos[3 * j + 1] - py;
            const double dz = pos[3 * j + 2] - pz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            s += mass[j] / sqrt(r2);
        }
        phi[t] = s;
    }
}

/* core/solvers/gravity.py:29-36 kinetic_energy. */
double orc_kinetic_energy(const double *vel, const double *mass, int64_t n) {
    double ke = 0.0;
#pragma omp parallel for reduction(+ : ke)
    for (int64_t i = 0; i < n; ++i) {
        const double *v = vel + 3 * i;
        ke += 0.5 * mass[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    return ke;
}

/* core/solvers/gravity.py:39-57 potential_energy: -1/2 G sum_i m_i
 * sum_{j != i} m_j / sqrt(r2 + eps2). */
double orc_potential_energy(const double *pos, const double *mass, int64_t n,
                            double G, double eps2) {
    double pe = 0.0;
#pragma omp parallel for reduction(+ : pe) schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        double acc_i = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            if (j == i) continue;
            const double dx = pos[3 * j] - px;
            const double dy = pos[3 * j + 1] - py;
            const double dz = pos[3 * j + 2] - pz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            acc_i += mass[j] / sqrt(r2);
        }
        pe += -0.5 * G * mass[i] * acc_i;
    }
    return pe;
}

/* core/integrators/leapfrog.py:11-22 in the order of core/engine.py:108-116:
 * kick(dt/2) -> drift(dt) -> acc -> kick(dt/2); acc holds the previous
 * step's accelerations on entry (primed by load_state, core/engine.py:81). */
void orc_kdk_direct(double *pos, double *vel, double *acc, const double *mass,
                    int64_t n, double G, double eps2, double dt,
                    int64_t nsteps) {
    const double half = 0.5 * dt;
    for (int64_t s = 0; s < nsteps; ++s) {
        for (int64_t k = 0; k < 3 * n; ++k) vel[k] += acc[k] * half;
        for (int64_t k = 0; k < 3 * n; ++k) pos[k] += vel[k] * dt;
        orc_direct_acc(pos, mass, acc, n, G, eps2);
        for (int64_t k = 0; k < 3 * n; ++k) vel[k] += acc[k] * half;
    }
}

/* ----------------------------------------------------- analytic potential
 * The analytic galaxy potential of grav_analytic
 * (core/living_galaxy_engine.py:124-151) and add_analytic
 * (core/gas_disk_engine.py:54-81), added to av in the reference's order:
 * Miyamoto-Nagai disk, then the Hernquist (hern = 1) or Plummer halo, then
 * the softened central point mass when smbh > 0. */
static void analytic_add(const double *p, double G, double M_d, double a,
                         double b, double M_h, double a_h, int hern,
                         double smbh, double *av) {
    const double x = p[0], y = p[1], z = p[2];
    const double R2 = x * x + y * y;
    const double S = sqrt(z * z + b * b);
    const double aS = a + S;
    const double invD3 = pow(R2 + aS * aS, -1.5);
    const double gmd = -G * M_d;
    av[0] += gmd * x * invD3;
    av[1] += gmd * y * invD3;
    av[2] += gmd * z * aS * invD3 / S;
    if (hern == 1) {
        const double r = sqrt(x * x + y * y + z * z);
        const double rs = r > 1e-6 ? r : 1e-6;
        const double c = -(G * M_h / (pow(rs + a_h, 2.0) * rs));
        av[0] += c * x;
        av[1] += c * y;
        av[2] += c * z;
    } else {
        const double rh = R2 + z * z + a_h * a_h;
        const double c = -(G * M_h * pow(rh, -1.5));
        av[0] += c * x;
        av[1] += c * y;
        av[2] += c * z;
    }
    if (smbh > 0.0) {
        const double rs = sqrt(x * x + y * y + z * z) + 1e-6;
        const double c = -(G * smbh / (rs * rs * rs));
        av[0] += c * x;
        av[1] += c * y;
        av[2] += c * z;
    }
}

/* grav_analytic / add_analytic: acc[i] += av (analytic part only). */
void orc_analytic_acc(const double *pos, double *acc, int64_t n, double G,
                      double M_d, double a, double b, double M_h, double a_h,
                      int hern, double smbh) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double av[3] = {0.0, 0.0, 0.0};
        analytic_add(pos + 3 * i, G, M_d, a, b, M_h, a_h, hern, smbh, av);
        for (int k = 0; k < 3; ++k) acc[3 * i + k] += av[k];
    }
}

/* add_grav_ext (core/gas_disk_engine.py:20-51): av = softened direct
 * self-gravity over all j (as compute_acc_direct), then the analytic terms,
 * then acc[i] += av. */
void orc_grav_ext_acc(const double *pos, const double *mass, double *acc,
                      int64_t n, double G, double eps2, double M_d, double a,
                      double b, double M_h, double a_h, int hern,
                      double smbh) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double av[3];
        direct_one(pos, mass, n, G, eps2, i, av);
        analytic_add(pos + 3 * i, G, M_d, a, b, M_h, a_h, hern, smbh, av);
        for (int k = 0; k < 3; ++k) acc[3 * i + k] += av[k];
    }
}

/* ------------------------------------------------------------------ Morton
 * core/solvers/barnes_hut.py:27-46.  lo = per-axis min, span = the largest
 * per-axis extent (1.0 if not > 0), scale = (2^bits-1)/(span*1.0000001),
 * q = clip((x-lo)*scale, 0, 2^bits-1) truncated to an integer, key =
 * interleave(qx, qy, qz) with x in bit 3k, y in 3k+1, z in 3k+2. */
static uint64_t spread3(uint64_t v, int bits) {
    uint64_t r = 0;
    for (int b = 0; b < bits; ++b) r |= ((v >> b) & 1ull) << (3 * b);
    return r;
}

void orc_morton(const double *pos, int64_t n, int bits, uint64_t *codes,
                double *lo_out, double *scale_out) {
    double lo[3] = {INFINITY, INFINITY, INFINITY};
    double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const double v = pos[3 * i + k];
            if (v < lo[k]) lo[k] = v;
            if (v > hi[k]) hi[k] = v;
        }
    double span = hi[0] - lo[0];
    for (int k = 1; k < 3; ++k)
        if (hi[k] - lo[k] > span) span = hi[k] - lo[k];
    if (!(span > 0)) span = 1.0;
    const double qmax = (double)((1ull << bits) - 1ull);
    const double scale = qmax / (span * 1.0000001);
    for (int64_t i = 0; i < n; ++i) {
        uint64_t q[3];
        for (int k = 0; k < 3; ++k) {
            double t = (pos[3 * i + k] - lo[k]) * scale;
            if (t < 0.0) t = 0.0;
            if (t > qmax) t = qmax;
            q[k] = (uint64_t)t;
        }
        codes[i] = spread3(q[0], bits) | (spread3(q[1], bits) << 1) |
                   (spread3(q[2], bits) << 2);
    }
    if (lo_out) memcpy(lo_out, lo, sizeof(lo));
    if (scale_out) *scale_out = scale;
}

/* Stable argsort of unsigned 64-bit keys (np.argsort(kind="stable"),
 * core/solvers/barnes_hut.py:247): LSD radix, 16-bit digits. */
void orc_stable_argsort_u64(const uint64_t *keys, int64_t n, int32_t *order) {
    int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    size_t *cnt = (size_t *)malloc(sizeof(size_t) * 65537);
    for (int64_t i = 0; i < n; ++i) order[i] = (int32_t)i;
    uint64_t all_or = 0;
    for (int64_t i = 0; i < n; ++i) all_or |= keys[i];
    int32_t *src = order, *dst = tmp;
    for (int shift = 0; shift < 64; shift += 16) {
        if (((all_or >> shift) & 0xFFFFull) == 0) continue;
        memset(cnt, 0, sizeof(size_t) * 65537);
        for (int64_t i = 0; i < n; ++i) cnt[((keys[src[i]] >> shift) & 0xFFFF) + 1]++;
        for (int d = 0; d < 65536; ++d) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n; ++i) dst[cnt[(keys[src[i]] >> shift) & 0xFFFF]++] = src[i];
        int32_t *t = src; src = dst; dst = t;
    }
    if (src != order) memcpy(order, src, sizeof(int32_t) * (size_t)n);
    free(tmp);
    free(cnt);
}

/* ------------------------------------------------------------- Karras build
 * core/solvers/barnes_hut.py:50-81: common-prefix length over bits 62..0 of
 * the codes; equal codes fall back to 63 + the prefix of the indices over
 * bits 30..0; -1 when j is out of range. */
static int clz63(uint64_t x) {
    int c = 0;
    for (uint64_t m = 1ull << 62; m && !(x & m); m >>= 1) ++c;
    return c;
}

static int clz31(uint32_t x) {
    int c = 0;
    for (uint32_t m = 1u << 30; m && !(x & m); m >>= 1) ++c;
    return c;
}

static int delta(int i, int j, int n, const int64_t *code) {
    if (j < 0 || j >= n) return -1;
    const uint64_t x = (uint64_t)(code[i] ^ code[j]);
    if (x == 0) return 63 + clz31((uint32_t)(i ^ j));
    return clz63(x);
}

/* core/solvers/barnes_hut.py:84-121 _build_radix (Karras 2012): internal
 * nodes 0..n-2; children stored as leaf id (< n) or internal id + n;
 * parent[] must be pre-filled with -1 by the caller (:250). */
void orc_build_radix(const int64_t *code, int n, int32_t *left, int32_t *right,
                     int32_t *parent) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n - 1; ++i) {
        const int d = delta(i, i + 1, n, code) > delta(i, i - 1, n, code) ? 1 : -1;
        const int d_min = delta(i, i - d, n, code);
        int l_max = 2;
        while (delta(i, i + l_max * d, n, code) > d_min) l_max *= 2;
        int l = 0;
        for (int t = l_max / 2; t >= 1; t /= 2)
            if (delta(i, i + (l + t) * d, n, code) > d_min) l += t;
        const int j = i + l * d;
        const int d_node = delta(i, j, n, code);
        int s = 0;
        int t2 = (l + 1) / 2;
        while (t2 >= 1) {
            if (delta(i, i + (s + t2) * d, n, code) > d_node) s += t2;
            t2 = t2 > 1 ? (t2 + 1) / 2 : 0;
        }
        const int gamma = i + s * d + (d < 0 ? d : 0);
        const int lo = i < j ? i : j;
        const int hi = i < j ? j : i;
        const int lc = (lo == gamma) ? gamma : gamma + n;
        const int rc = (hi == gamma + 1) ? gamma + 1 : gamma + 1 + n;
        left[i] = lc;
        right[i] = rc;
        parent[lc] = i + n;
        parent[rc] = i + n;
    }
}

/* -------------------------------------------------------- node summaries
 * core/solvers/barnes_hut.py:124-177: leaf com/mass/AABB from the sorted
 * particle; every leaf adds its mass, mass*position and AABB into each
 * ancestor (here in leaf order, serially); internal com = moment / mass. */
void orc_summaries(const int32_t *order, const double *pos, const double *mass,
                   const int32_t *parent, int n, double *com, double *nmass,
                   double *nmin, double *nmax) {
    const int m = 2 * n - 1;
    double *nmom = (double *)calloc((size_t)(3 * (m > 0 ? m : 1)), sizeof(double));
    for (int li = 0; li < n; ++li) {
        const int p = order[li];
        for (int k = 0; k < 3; ++k) {
            com[3 * li + k] = pos[3 * p + k];
            nmin[3 * li + k] = pos[3 * p + k];
            nmax[3 * li + k] = pos[3 * p + k];
        }
        nmass[li] = mass[p];
    }
    for (int ii = 0; ii < n - 1; ++ii) {
        const int node = ii + n;
        nmass[node] = 0.0;
        for (int k = 0; k < 3; ++k) {
            com[3 * node + k] = 0.0;
            nmin[3 * node + k] = 1e30;
            nmax[3 * node + k] = -1e30;
        }
    }
    for (int li = 0; li < n; ++li) {
        const double mm = nmass[li];
        const double *pp = com + 3 * li;
        for (int node = parent[li]; node >= 0; node = parent[node]) {
            nmass[node] += mm;
            for (int k = 0; k < 3; ++k) {
                nmom[3 * node + k] += mm * pp[k];
                if (pp[k] < nmin[3 * node + k]) nmin[3 * node + k] = pp[k];
                if (pp[k] > nmax[3 * node + k]) nmax[3 * node + k] = pp[k];
            }
        }
    }
    for (int ii = 0; ii < n - 1; ++ii) {
        const int node = ii + n;
        const double mm = nmass[node];
        if (mm > 0.0)
            for (int k = 0; k < 3; ++k) com[3 * node + k] = nmom[3 * node + k] / mm;
    }
    free(nmom);
}

/* ---------------------------------------------------------------- traverse
 * core/solvers/barnes_hut.py:180-217 _traverse for particle p: DFS from the
 * root with an explicit stack; a leaf adds its monopole unless it is p
 * itself; an internal node is accepted when size^2 < theta2 * (|d|^2+eps2)
 * (size = largest AABB extent), else both children are pushed (left, then
 * right; right is popped first) when sp + 2 <= max_stack, and silently
 * dropped otherwise.  Returns the number of dropped pushes for p. */
static int64_t traverse_one(const double *pos, const int32_t *order,
                            const double *com, const double *nmass,
                            const double *nmin, const double *nmax,
                            const int32_t *left, const int32_t *right, int n,
                            int root, double theta2, double eps2, int max_stack,
                            double G, int p, int32_t *stack, double *out,
                            double *phi_out) {
    const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
    double ax = 0.0, ay = 0.0, az = 0.0, w = 0.0;
    int64_t dropped = 0;
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const int node = stack[--sp];
        if (node < n) {
            if (order[node] != p) {
                const double dx = com[3 * node] - px;
                const double dy = com[3 * node + 1] - py;
                const double dz = com[3 * node + 2] - pz;
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                const double inv = 1.0 / sqrt(r2);
                const double s = G * nmass[node] * inv * inv * inv;
                ax += s * dx;
                ay += s * dy;
                az += s * dz;
                w += nmass[node] * inv;
            }
        } else {
            const int ii = node - n;
            const double dx = com[3 * node] - px;
            const double dy = com[3 * node + 1] - py;
            const double dz = com[3 * node + 2] - pz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double size = nmax[3 * node] - nmin[3 * node];
            for (int k = 1; k < 3; ++k) {
                const double e = nmax[3 * node + k] - nmin[3 * node + k];
                if (e > size) size = e;
            }
            if (size * size < theta2 * r2) {
                const double inv = 1.0 / sqrt(r2);
                const double s = G * nmass[node] * inv * inv * inv;
                ax += s * dx;
                ay += s * dy;
                az += s * dz;
                w += nmass[node] * inv;
            } else if (sp + 2 <= max_stack) {
                stack[sp++] = left[ii];
                stack[sp++] = right[ii];
            } else {
                ++dropped;
            }
        }
    }
    out[0] = ax;
    out[1] = ay;
    out[2] = az;
    if (phi_out) *phi_out = w;
    return dropped;
}

/* Evaluate the traversal for the given particles (all when targets == NULL).
 * acc is indexed like targets (or by particle when targets == NULL). */
/* phi (optional): the tree potential sum of each target, sum m / sqrt(r2)
 * over the nodes the walk above accepts (the own leaf skipped, no G): the
 * potential_energy sum (core/solvers/gravity.py:47-55) evaluated on the
 * reference traversal's node set, the check for a device tree potential. */
int64_t orc_traverse_phi(const double *pos, const int32_t *order, const double *com,
                         const double *nmass, const double *nmin,
                         const double *nmax, const int32_t *left,
                         const int32_t *right, int n, double theta2, double eps2,
                         int max_stack, double G, const int64_t *targets,
                         int64_t nt, double *acc, double *phi);

int64_t orc_traverse(const double *pos, const int32_t *order, const double *com,
                     const double *nmass, const double *nmin,
                     const double *nmax, const int32_t *left,
                     const int32_t *right, int n, double theta2, double eps2,
                     int max_stack, double G, const int64_t *targets,
                     int64_t nt, double *acc) {
    return orc_traverse_phi(pos, order, com, nmass, nmin, nmax, left, right, n, theta2, eps2,
                            max_stack, G, targets, nt, acc, NULL);
}

int64_t orc_traverse_phi(const double *pos, const int32_t *order, const double *com,
                         const double *nmass, const double *nmin,
                         const double *nmax, const int32_t *left,
                         const int32_t *right, int n, double theta2, double eps2,
                         int max_stack, double G, const int64_t *targets,
                         int64_t nt, double *acc, double *phi) {
    int64_t dropped = 0;
    const int64_t count = targets ? nt : n;
#pragma omp parallel reduction(+ : dropped)
    {
        int32_t *stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)(max_stack > 0 ? max_stack : 1));
#pragma omp for schedule(dynamic, 64)
        for (int64_t t = 0; t < count; ++t) {
            const int p = targets ? (int)targets[t] : (int)t;
            dropped += traverse_one(pos, order, com, nmass, nmin, nmax, left,
                                    right, n, n, theta2, eps2, max_stack, G, p,
                                    stack, acc + 3 * t, phi ? phi + t : NULL);
        }
        free(stack);
    }
    return dropped;
}

/* Group walk: the targets are cut into groups, the maximal subtrees with at
 * most `group` leaves (consecutive ranges of the key order, each inside one
 * node's box); a group accepts a node when size^2 < theta2 (dmin^2 + eps2),
 * dmin the distance from the node's centre of mass to the group's bounding
 * box, and every leaf (its own included) is accepted.  Each target of the
 * group sums the accepted nodes' monopoles (acc with G, phi without G, its
 * own leaf skipped): the FP64 restatement of the device's group traversal,
 * with the reference's acceptance test (core/solvers/barnes_hut.py:204-210)
 * applied to a box instead of a point.  acc / phi are indexed by particle. */
static void group_walk_one(const double *pos, const int32_t *order, const double *com,
                           const double *nmass, const double *nmin, const double *nmax,
                           const int32_t *left, const int32_t *right, int n, int b0, int b1,
                           double theta2, double eps2, double G, int32_t *stack, int32_t *list,
                           double *acc, double *phi) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = b0; i < b1; ++i)
        for (int a = 0; a < 3; ++a) {
            const double x = pos[3 * order[i] + a];
            if (x < lo[a]) lo[a] = x;
            if (x > hi[a]) hi[a] = x;
        }
    int sp = 0, nl = 0;
    if (n >= 2) stack[sp++] = n; else list[nl++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        if (node < n) {
            list[nl++] = node;
            continue;
        }
        double d2 = 0.0, size = 0.0;
        for (int a = 0; a < 3; ++a) {
            const double c = com[3 * node + a];
            double d = lo[a] - c > c - hi[a] ? lo[a] - c : c - hi[a];
            d = d > 0.0 ? d : 0.0;
            d2 += d * d;
            const double e = nmax[3 * node + a] - nmin[3 * node + a];
            if (e > size) size = e;
        }
        if (size * size < theta2 * (d2 + eps2)) {
            list[nl++] = node;
        } else {
            stack[sp++] = left[node - n];
            stack[sp++] = right[node - n];
        }
    }
    for (int i = b0; i < b1; ++i) {
        const int p = order[i];
        const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
        double ax = 0.0, ay = 0.0, az = 0.0, w = 0.0;
        for (int t = 0; t < nl; ++t) {
            const int node = list[t];
            if (node < n && order[node] == p) continue;
            const double dx = com[3 * node] - px;
            const double dy = com[3 * node + 1] - py;
            const double dz = com[3 * node + 2] - pz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double inv = 1.0 / sqrt(r2);
            const double sc = G * nmass[node] * inv * inv * inv;
            ax += sc * dx;
            ay += sc * dy;
            az += sc * dz;
            w += nmass[node] * inv;
        }
        acc[3 * p] = ax;
        acc[3 * p + 1] = ay;
        acc[3 * p + 2] = az;
        if (phi) phi[p] = w;
    }
}

void orc_group_walk(const double *pos, const int32_t *order, const double *com,
                    const double *nmass, const double *nmin, const double *nmax,
                    const int32_t *left, const int32_t *right, int n, int group,
                    double theta2, double eps2, double G, double *acc,
                    double *phi) {
    /* The groups: descend from the root until a node has at most `group`
     * leaves (its leaves are its leftmost to its rightmost leaf). */
    int32_t *g0 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t *g1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t *st = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * n + 2));
    int ng = 0, sp = 0;
    st[sp++] = n >= 2 ? n : 0;
    while (sp > 0) {
        const int v = st[--sp];
        int lo = v, hi = v;
        if (v >= n) {
            lo = v;
            while (lo >= n) lo = left[lo - n];
            hi = v;
            while (hi >= n) hi = right[hi - n];
        }
        if (hi - lo + 1 <= group) {
            g0[ng] = lo;
            g1[ng] = hi + 1;
            ++ng;
        } else {
            st[sp++] = right[v - n];
            st[sp++] = left[v - n];
        }
    }
    free(st);
#pragma omp parallel
    {
        int32_t *stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * n + 2));
        int32_t *list = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * n + 2));
#pragma omp for schedule(dynamic, 4)
        for (int g = 0; g < ng; ++g)
            group_walk_one(pos, order, com, nmass, nmin, nmax, left, right, n, g0[g], g1[g], theta2,
                           eps2, G, stack, list, acc, phi);
        free(stack);
        free(list);
    }
    free(g0);
    free(g1);
}

/* ------------------------------------------------------- neighbour grid
 * NeighborGrid.rebuild / rebuild_all (core/solvers/neighbor_grid.py:49-136):
 * gas = particles with is_star == 0 (all when is_star is NULL), in index
 * order; cell = max(2 h_max, min_radius), 1 if not > 1e-9; lo / span from
 * the gas positions; dims = max(int64(floor(span / cell)) + 1, 1), the cell
 * grown by 1.3 while prod(dims) > max_cells; key = (i dy + j) dz + k with
 * ijk = clip(int64((x - lo) / cell), 0, dims - 1); gsort = gas in stable key
 * order (zero-padded to n), cell_start = exclusive prefix of the per-cell
 * counts (n_cells + 1 entries, zero above).  Returns ngas; with no gas the
 * outputs are left untouched.  int64 casts follow numpy on x86-64
 * (truncation, INT64_MIN for NaN and out-of-range values). */
static int64_t np_i64(double t) {
    if (!(t < 9223372036854775808.0 && t > -9223372036854775808.0)) return INT64_MIN;
    return (int64_t)t;
}

int64_t orc_grid_rebuild(const double *pos, const double *h, const int32_t *is_star,
                         int64_t n, double min_radius, int64_t max_cells,
                         int32_t *gsort, int32_t *cell_start, int64_t *dims_out,
                         double *lo_out, double *inv_cell_out) {
    int64_t ngas = 0;
    for (int64_t i = 0; i < n; ++i) ngas += (!is_star || is_star[i] == 0);
    if (ngas == 0) return 0;
    int32_t *gas = (int32_t *)malloc(sizeof(int32_t) * (size_t)ngas);
    double hmax = -INFINITY, lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    int64_t g = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (is_star && is_star[i] != 0) continue;
        gas[g++] = (int32_t)i;
        if (h[i] > hmax) hmax = h[i];
        for (int a = 0; a < 3; ++a) {
            const double x = pos[3 * i + a];
            if (x < lo[a]) lo[a] = x;
            if (x > hi[a]) hi[a] = x;
        }
    }
    double cell = 2.0 * hmax > min_radius ? 2.0 * hmax : min_radius;
    cell = cell > 1e-9 ? cell : 1.0;
    double span[3];
    for (int a = 0; a < 3; ++a) span[a] = hi[a] - lo[a];
    int64_t dims[3];
    for (;;) {
        for (int a = 0; a < 3; ++a) {
            const int64_t f = np_i64(floor(span[a] / cell));
            dims[a] = (f != INT64_MIN && f + 1 > 1) ? f + 1 : 1;
        }
        if ((double)dims[0] * (double)dims[1] * (double)dims[2] <= (double)max_cells) break;
        cell *= 1.3;
    }
    const int64_t n_cells = dims[0] * dims[1] * dims[2];
    int64_t *key = (int64_t *)malloc(sizeof(int64_t) * (size_t)ngas);
    int64_t *cnt = (int64_t *)calloc((size_t)n_cells + 1, sizeof(int64_t));
    for (int64_t p = 0; p < ngas; ++p) {
        const int64_t i = gas[p];
        int64_t q[3];
        for (int a = 0; a < 3; ++a) {
            int64_t v = np_i64((pos[3 * i + a] - lo[a]) / cell);
            q[a] = v < 0 ? 0 : (v > dims[a] - 1 ? dims[a] - 1 : v);
        }
        key[p] = (q[0] * dims[1] + q[1]) * dims[2] + q[2];
        cnt[key[p] + 1] += 1;
    }
    for (int64_t c = 0; c <= max_cells; ++c) cell_start[c] = 0;
    for (int64_t c = 0; c < n_cells; ++c) cnt[c + 1] += cnt[c];
    for (int64_t c = 0; c <= n_cells; ++c) cell_start[c] = (int32_t)cnt[c];
    for (int64_t p = 0; p < ngas; ++p) gsort[cnt[key[p]]++] = gas[p]; /* stable */
    for (int64_t p = ngas; p < n; ++p) gsort[p] = 0;
    for (int a = 0; a < 3; ++a) {
        dims_out[a] = dims[a];
        lo_out[a] = lo[a];
    }
    *inv_cell_out = 1.0 / cell;
    free(gas);
    free(key);
    free(cnt);
    return ngas;
}
