// nb_md.cu -- device-resident molecular dynamics around the nonbonded evaluation: leapfrog
// steps with rigid three-site waters, and the DCD trajectory writer.
//
// MOIL's integrator (dynamics/dyna.f:183-330) advances positions with leapfrog and holds
// water geometry with SHAKE (dynamics/shakept.f, matrix SHAKE dynamics/mshakpt.f); velocity
// constraints follow (dynamics/shakevl.f).  Here, after each evaluation,
//     v(t + dt/2) = v(t - dt/2) - dt * c * dpot / m          (c = 418.4: kcal/mol/Å/amu -> Å/ps^2)
//     x(t + dt)   = SETTLE(x(t), x(t) + dt * v(t + dt/2)),   v(t + dt/2) = (x(t + dt) - x(t)) / dt
// with SETTLE the analytic rigid-water solution of Miyamoto and Kollman (J. Comput. Chem. 13,
// 952 (1992)): the unconstrained molecule is expressed in a frame built from the previous
// molecule, the rotations phi, psi (out of plane) and theta (in plane) place the rigid
// molecule keeping the centre of mass and constraint forces along the old bonds.  Atoms
// outside waters move unconstrained (this library holds no bonded terms).  FP64 throughout.
// The trajectory writer follows dynamics/wdyncrd.f's binary branch: Fortran unformatted
// sequential records (4-byte length before and after each record).
#include <cstdio>
#include <cstring>

#include "nb_internal.h"

namespace {

constexpr double kAccel = 418.4;

__device__ __forceinline__ double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ void cross3(const double *a, const double *b, double *c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ void unit3(double *a)
{
    const double s = 1.0 / sqrt(dot3(a, a));
    a[0] *= s; a[1] *= s; a[2] *= s;
}

// rigid positions p1[3][3] (O, H, H) from the previous rigid p0 and the unconstrained p1;
// doh, dhh the rigid distances, mo, mh the masses
__device__ void settle(const double p0[3][3], double p1[3][3], double doh, double dhh, double mo, double mh)
{
    const double mt = mo + 2.0 * mh, rc = 0.5 * dhh, h = sqrt(doh * doh - rc * rc);
    const double ra = 2.0 * mh * h / mt, rb = h - ra;
    double com[3], a1[3], b1[3], c1[3], ab0[3], ac0[3], ex[3], ey[3], ez[3];
    for (int d = 0; d < 3; ++d) {
        com[d] = (mo * p1[0][d] + mh * (p1[1][d] + p1[2][d])) / mt;
        a1[d] = p1[0][d] - com[d];
        b1[d] = p1[1][d] - com[d];
        c1[d] = p1[2][d] - com[d];
        ab0[d] = p0[1][d] - p0[0][d];
        ac0[d] = p0[2][d] - p0[0][d];
    }
    // frame: z normal to the previous molecule, x normal to z and the new O offset
    cross3(ab0, ac0, ez);
    cross3(a1, ez, ex);
    cross3(ez, ex, ey);
    unit3(ex); unit3(ey); unit3(ez);
    const double xb0 = dot3(ab0, ex), yb0 = dot3(ab0, ey), xc0 = dot3(ac0, ex), yc0 = dot3(ac0, ey);
    const double za1 = dot3(a1, ez);
    const double xb1 = dot3(b1, ex), yb1 = dot3(b1, ey), zb1 = dot3(b1, ez);
    const double xc1 = dot3(c1, ex), yc1 = dot3(c1, ey), zc1 = dot3(c1, ez);
    // phi and psi: the out-of-plane heights of O and of the H-H axis are kept
    const double sphi = za1 / ra, cphi = sqrt(fmax(1.0 - sphi * sphi, 0.0));
    const double spsi = (zb1 - zc1) / (2.0 * rc * cphi), cpsi = sqrt(fmax(1.0 - spsi * spsi, 0.0));
    const double ya2 = ra * cphi, xb2 = -rc * cpsi;
    const double yb2 = -rb * cphi - rc * spsi * sphi, yc2 = -rb * cphi + rc * spsi * sphi;
    // theta: the in-plane rotation for which the constraint forces lie along the old bonds
    const double al = xb2 * (xb0 - xc0) + yb0 * yb2 + yc0 * yc2;
    const double be = xb2 * (yc0 - yb0) + xb0 * yb2 + xc0 * yc2;
    const double ga = xb0 * yb1 - xb1 * yb0 + xc0 * yc1 - xc1 * yc0;
    const double ab2 = al * al + be * be;
    const double sth = (al * ga - be * sqrt(fmax(ab2 - ga * ga, 0.0))) / ab2, cth = sqrt(fmax(1.0 - sth * sth, 0.0));
    const double loc[3][3] = {{-ya2 * sth, ya2 * cth, za1},
                              {xb2 * cth - yb2 * sth, xb2 * sth + yb2 * cth, zb1},
                              {-xb2 * cth - yc2 * sth, -xb2 * sth + yc2 * cth, zc1}};
    for (int m = 0; m < 3; ++m)
        for (int d = 0; d < 3; ++d) p1[m][d] = com[d] + loc[m][0] * ex[d] + loc[m][1] * ey[d] + loc[m][2] * ez[d];
}

// one water per thread: its caller atoms are consecutive (O, H, H)
__global__ void k_leapfrog_water(int nW, const int *__restrict__ unit_atom, const double *__restrict__ mass,
                                 double dt, double doh, double dhh, double *__restrict__ coor,
                                 double *__restrict__ vel, const double *__restrict__ dpot)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nW) return;
    const size_t a = (size_t)unit_atom[w];
    double p0[3][3], p1[3][3];
    for (int m = 0; m < 3; ++m) {
        const double f = dt * kAccel / mass[a + m];
        for (int d = 0; d < 3; ++d) {
            const size_t k = 3 * (a + m) + d;
            p0[m][d] = coor[k];
            p1[m][d] = p0[m][d] + dt * (vel[k] - f * dpot[k]);
        }
    }
    settle(p0, p1, doh, dhh, mass[a], mass[a + 1]);
    const double inv = 1.0 / dt;
    for (int m = 0; m < 3; ++m)
        for (int d = 0; d < 3; ++d) {
            const size_t k = 3 * (a + m) + d;
            vel[k] = (p1[m][d] - p0[m][d]) * inv;
            coor[k] = p1[m][d];
        }
}

// every atom outside a water, unconstrained
__global__ void k_leapfrog_free(int natom, const unsigned *__restrict__ aflags, const double *__restrict__ mass,
                                double dt, double *__restrict__ coor, double *__restrict__ vel,
                                const double *__restrict__ dpot)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natom || (aflags[a] & SF_WATER)) return;
    const double f = dt * kAccel / mass[a];
    for (int d = 0; d < 3; ++d) {
        const size_t k = 3 * (size_t)a + d;
        vel[k] -= f * dpot[k];
        coor[k] += dt * vel[k];
    }
}

// kinetic energy partial sums per block (fixed order), summed on the host
__global__ void __launch_bounds__(256) k_kinetic(int natom, const double *__restrict__ mass,
                                                 const double *__restrict__ vel, double *__restrict__ part)
{
    __shared__ double sh[256];
    double s = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < natom; a += gridDim.x * blockDim.x) {
        const double *v = vel + 3 * (size_t)a;
        s += 0.5 * mass[a] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0] / kAccel;
}

// Step control of the device-side step loop (d_mdctl = {evaluations since the last rebuild,
// rebuild requested, sticky error bits}).  Before an evaluation: the status words the host
// writes before a normal evaluation, with the rebuild forced when the list period is reached
// or a rebuild was requested (the skin check of the coordinate preparation adds its own).
__global__ void k_md_begin(int *__restrict__ st, int *__restrict__ ctl, int list_period)
{
    st[0] = (ctl[1] || (list_period > 0 && ctl[0] >= list_period)) ? 1 : 0;
    for (int k = 1; k < 8; ++k) st[k] = 0;
    ctl[1] = 0;
}
// the gate of a step: its body runs only while no step of the call has raised an error (after
// one, the call is redone from its starting state by the per-step path)
__global__ void k_md_gate(cudaGraphConditionalHandle h, const int *__restrict__ ctl)
{
    cudaGraphSetConditional(h, ctl[2] == 0 ? 1u : 0u);
}
// after it: the error bits kept across steps, the rebuild counter advanced
__global__ void k_md_end(const int *__restrict__ st, int *__restrict__ ctl)
{
    if (st[0]) ctl[0] = 0;
    ctl[0] += 1;
    ctl[2] |= st[1];
}

// the integrator kernels of one (ungrouped) context over its caller-atom range
int integrate(NbCtx *c, cudaStream_t s, double *coor, double *vel, const double *mass, const double *dpot,
              double dt, double doh, double dhh)
{
    if (c->nW > 0)
        k_leapfrog_water<<<(int)((c->nW + 127) / 128), 128, 0, s>>>((int)c->nW, c->d_unit_atom, mass, dt, doh, dhh,
                                                                    coor, vel, dpot);
    if (c->nA > 0)
        k_leapfrog_free<<<(int)((c->natom + 255) / 256), 256, 0, s>>>((int)c->natom, c->d_aflags, mass, dt, coor,
                                                                      vel, dpot);
    NB_CUDA_OK(c, cudaGetLastError());
    return MOIL_NB_OK;
}

}  // namespace

void nb_launch_md_begin(NbCtx *c, cudaStream_t s)
{
    k_md_begin<<<1, 1, 0, s>>>(c->d_status, c->d_mdctl, c->list_period);
    c->launches++;
}

void nb_launch_md_gate(NbCtx *c, cudaStream_t s, cudaGraphConditionalHandle h)
{
    k_md_gate<<<1, 1, 0, s>>>(h, c->d_mdctl);
    c->launches++;
}

void nb_launch_md_end(NbCtx *c, cudaStream_t s)
{
    k_md_end<<<1, 1, 0, s>>>(c->d_status, c->d_mdctl);
    c->launches++;
}

int nb_launch_integrate(NbCtx *c, cudaStream_t s, double *coor, double *vel, const double *mass, const double *dpot,
                        double dt, double doh, double dhh)
{
    return integrate(c, s, coor, vel, mass, dpot, dt, doh, dhh);
}

namespace {

void put_record(FILE *f, const void *data, uint32_t bytes)
{
    fwrite(&bytes, 4, 1, f);
    fwrite(data, 1, bytes, f);
    fwrite(&bytes, 4, 1, f);
}

}  // namespace

extern "C" {

int moil_nb_md_step(moil_nb_ctx *h, double *d_coor, double *d_vel, const double *d_mass, double dt, int nsteps,
                    const double *water_geom, moil_energies *energies, double *ekin)
{
    if (!h || !d_coor || !d_vel || !d_mass || !(dt > 0.0) || nsteps < 0) return MOIL_NB_ERR_ARG;
    if (!h->inited || h->pending) return MOIL_NB_ERR_STATE;
    cudaSetDevice(h->device);
    // TIP3P: O-H 0.9572 Å, H-O-H 104.52 degrees
    const double doh = water_geom ? water_geom[0] : 0.9572;
    const double dhh = water_geom ? water_geom[1] : 2.0 * 0.9572 * sin(104.52 * M_PI / 360.0);
    const size_t n = (size_t)h->natom;
    if (!h->d_md_dpot) NB_CUDA_OK(h, cudaMalloc(&h->d_md_dpot, sizeof(double) * 3 * std::max<size_t>(n, 1)));
    // Device-side loop: every context replays a graph of whole steps nsteps times with no host
    // wait between them; the error bits are read once at the end.  Any error (a list overflow
    // to regrow, a non-finite coordinate) sends the call back to the saved state and through
    // the per-step path below, which handles it as a single evaluation does.
    int first = 0;
    const bool loop = nsteps > 1 && h->use_graph && !h->timing;
    if (loop) {
        if (!h->d_md_save) NB_CUDA_OK(h, cudaMalloc(&h->d_md_save, sizeof(double) * 6 * std::max<size_t>(n, 1)));
        NB_CUDA_OK(h, cudaMemcpyAsync(h->d_md_save, d_coor, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, h->stream));
        NB_CUDA_OK(h, cudaMemcpyAsync(h->d_md_save + 3 * n, d_vel, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice,
                                      h->stream));
        std::vector<NbCtx *> ctxs;
        if (h->grp.empty()) ctxs.push_back(h);
        else for (NbCtx *c : h->grp) ctxs.push_back(c);
        int rc = MOIL_NB_OK;
        for (size_t g = 0; g < ctxs.size() && rc == MOIL_NB_OK; ++g) {
            NbCtx *c = ctxs[g];
            const int64_t a0 = h->grp.empty() ? 0 : h->grp_atom0[g];
            if (c != h) {
                NB_CUDA_OK(h, cudaEventRecord(h->ev[11], h->stream));            // the snapshot copies
                NB_CUDA_OK(h, cudaStreamWaitEvent(c->stream, h->ev[11], 0));
            }
            rc = nb_md_loop(c, d_coor + 3 * a0, d_vel + 3 * a0, d_mass + a0, h->d_md_dpot + 3 * a0, dt, doh, dhh,
                            nsteps);
        }
        int err = 0;
        for (NbCtx *c : ctxs) {
            NB_CUDA_OK(h, cudaStreamSynchronize(c->stream));
            if (rc == MOIL_NB_OK) {
                err |= c->h_status[22];
                if (!c->h_status[22]) {
                    // the host's view of the list schedule, pair counts and energies
                    c->evals_since_build = c->h_status[20];
                    c->need_rebuild = 0;
                    read_energies_of(c, nullptr);
                }
            }
        }
        if (rc == MOIL_NB_OK && !err) {
            if (!h->grp.empty()) {
                h->last_site_pairs = 0;
                for (NbCtx *c : ctxs) h->last_site_pairs += c->last_site_pairs;
            }
            if (energies) {
                for (size_t g = 0; g < ctxs.size(); ++g)
                    read_energies_of(ctxs[g], energies + (h->grp.empty() ? 0 : h->grp_rep0[g]));
            }
            first = nsteps;
        } else {
            NB_CUDA_OK(h, cudaMemcpyAsync(d_coor, h->d_md_save, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice,
                                          h->stream));
            NB_CUDA_OK(h, cudaMemcpyAsync(d_vel, h->d_md_save + 3 * n, sizeof(double) * 3 * n,
                                          cudaMemcpyDeviceToDevice, h->stream));
            NB_CUDA_OK(h, cudaStreamSynchronize(h->stream));
            for (NbCtx *c : ctxs) c->need_rebuild = 1;
            if (rc != MOIL_NB_OK) cudaGetLastError();
        }
    }
    for (int step = first; step < nsteps; ++step) {
        int rc = moil_nb_eval_device(h, d_coor, h->d_md_dpot, step + 1 == nsteps ? energies : nullptr);
        if (rc != MOIL_NB_OK) return rc;
        if (h->grp.empty()) {
            rc = integrate(h, h->stream, d_coor, d_vel, d_mass, h->d_md_dpot, dt, doh, dhh);
        } else {
            // each group integrates its own atoms on its stream; the handle's stream waits
            for (size_t g = 0; g < h->grp.size() && rc == MOIL_NB_OK; ++g) {
                const int64_t a0 = h->grp_atom0[g];
                rc = integrate(h->grp[g], h->grp[g]->stream, d_coor + 3 * a0, d_vel + 3 * a0, d_mass + a0,
                               h->d_md_dpot + 3 * a0, dt, doh, dhh);
            }
            for (NbCtx *c : h->grp) {
                NB_CUDA_OK(h, cudaEventRecord(c->ev[11], c->stream));
                NB_CUDA_OK(h, cudaStreamWaitEvent(h->stream, c->ev[11], 0));
            }
        }
        if (rc != MOIL_NB_OK) { if (h->err.empty() && !h->grp.empty()) h->err = h->grp[0]->err; return rc; }
    }
    if (ekin) {
        const int nb = (int)std::min<size_t>((n + 255) / 256, 1024);
        std::vector<double> part(std::max(nb, 1));
        double *d_part = nullptr;
        NB_CUDA_OK(h, cudaMallocAsync((void **)&d_part, sizeof(double) * part.size(), h->stream));
        k_kinetic<<<std::max(nb, 1), 256, 0, h->stream>>>((int)n, d_mass, d_vel, d_part);
        NB_CUDA_OK(h, cudaGetLastError());
        NB_CUDA_OK(h, cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                                      h->stream));
        NB_CUDA_OK(h, cudaFreeAsync(d_part, h->stream));
        NB_CUDA_OK(h, cudaStreamSynchronize(h->stream));
        double k = 0.0;
        for (double v : part) k += v;
        *ekin = k;
    } else {
        NB_CUDA_OK(h, cudaStreamSynchronize(h->stream));
    }
    return MOIL_NB_OK;
}

int moil_nb_dcd_write(const char *path, int first, int nframes, int natom, const double *coor)
{
    if (!path || natom <= 0 || !coor) return MOIL_NB_ERR_ARG;
    FILE *f = fopen(path, first ? "wb" : "ab");
    if (!f) return MOIL_NB_ERR_ARG;
    if (first) {
        // header as dynamics/wdyncrd.f writes it: 'CORD' + 20 integers (1: frames,
        // 9: fixed atoms), a title record, the atom count
        unsigned char rec[84];
        int32_t vari[20] = {0};
        vari[0] = nframes;
        memcpy(rec, "CORD", 4);
        memcpy(rec + 4, vari, sizeof vari);
        put_record(f, rec, 84);
        unsigned char title[84];
        const int32_t one = 1;
        memcpy(title, &one, 4);
        char text[80];
        memset(text, ' ', 80);
        const char *t = "A dummy title to dynamics coordinates";
        memcpy(text, t, strlen(t));
        memcpy(title + 4, text, 80);
        put_record(f, title, 84);
        const int32_t n = natom;
        put_record(f, &n, 4);
    }
    std::vector<float> v(natom);
    for (int d = 0; d < 3; ++d) {
        for (int a = 0; a < natom; ++a) v[a] = (float)coor[3 * (size_t)a + d];
        put_record(f, v.data(), (uint32_t)(sizeof(float) * natom));
    }
    const int bad = ferror(f);
    fclose(f);
    return bad ? MOIL_NB_ERR_ARG : MOIL_NB_OK;
}

}  // extern "C"
