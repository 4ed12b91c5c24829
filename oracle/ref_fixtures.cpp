/*
 * ref_fixtures.cpp - golden-vector generator that runs the REFERENCE's own code.
 *
 * Test infrastructure only.  Linked by oracle/Makefile against the reference's
 * sources where they lie (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu host
 * code, VortexState.cpp, and jukan_koodit Mesh/Types/Output); the binary is
 * written to oracle/_ref/ and run by tests/golden/make_golden.py, which commits
 * what it prints as fixtures under tests/golden/.  Nothing here is shipped.
 *
 * Sub-commands (argv[1]):
 *   tables   - getPositions()/getLaplacian() of GPUGrossPitaevskii_BCC.cu:73-142,
 *              with the byte offsets decoded into block offsets.
 *   mesh     - Hodge data of the reference Mesh library around interior nodes and
 *              bodies of DelaunayMesh::createBccGrid (DelaunayMesh.cpp:178-219,
 *              Mesh.cpp:1479-1512).
 *   vortex   - VortexState loaded from a state file (VortexState.cpp:49-72) and
 *              the diagnostics main() prints (GPUGrossPitaevskii_BCC.cu:503-548),
 *              psi samples, getPhase, and the Random(54363) noise stream.
 *   setup    - the host-side set-up of integrateInTime (GPUGrossPitaevskii_BCC.cu:
 *              222-348) for a caller-chosen block_scale, restated as a loop over
 *              the reference's own functions; arrays go to a binary file.
 */
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "koodit/GrossPitaevskii/VortexState.hpp"
#include "jukan_koodit/Types/Buffer.hpp"
#include "jukan_koodit/Types/Complex.hpp"
#include "jukan_koodit/Types/Random.hpp"
#include "jukan_koodit/Types/Vector3.hpp"
#include "jukan_koodit/Mesh/DelaunayMesh.hpp"

// Defined (non-static) in GPUGrossPitaevskii_BCC.cu.
extern ddouble RATIO;
extern ddouble KAPPA;
extern ddouble G;
// BLOCK_WIDTH (sqrt(8) per axis, GPUGrossPitaevskii_BCC.cu:70) and VOLUME
// (sqrt(32/9), :71) have internal linkage there; their values are restated.
static const Vector3 BLOCK_WIDTH = std::sqrt(8.0) * Vector3(1, 1, 1);
static const ddouble VOLUME = std::sqrt(32.0 / 9.0);
void getPositions(Buffer<Vector3> &pos);
ddouble getLaplacian(Buffer<int2> &ind, const int nx, const int ny, const int nz);
ddouble potentialV3(const Vector3 &p);

static void print_tables()
{
    Buffer<Vector3> pos;
    getPositions(pos);
    // Distinct strides so that every (dx,dy,dz) in {-1,0,1}^3 decodes uniquely.
    const int NX = 1, NY = 8, NZ = 64;
    Buffer<int2> ind;
    const double hodge = getLaplacian(ind, NX, NY, NZ);
    std::printf("{\n  \"source\": \"koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:69-142\",\n");
    std::printf("  \"hodge\": %.17g,\n", hodge);
    std::printf("  \"block_width\": %.17g,\n", BLOCK_WIDTH.x);
    std::printf("  \"volume\": %.17g,\n", VOLUME);
    std::printf("  \"positions\": [");
    for (uint i = 0; i < pos.size(); i++)
        std::printf("%s[%.17g, %.17g, %.17g]", i ? ", " : "", pos[i].x, pos[i].y, pos[i].z);
    std::printf("],\n  \"neighbours\": [");
    for (uint i = 0; i < ind.size(); i++) {
        int off = ind[i].x;
        int dz = (off + 32 + 64 * 2) / 64 - 2;  // off = dx + 8 dy + 64 dz, |dx|,|dy| <= 1
        int r = off - 64 * dz;
        int dy = (r + 4 + 8 * 2) / 8 - 2;
        int dx = r - 8 * dy;
        std::printf("%s[%d, %d, %d, %d]", i ? ", " : "", dx, dy, dz, ind[i].y);
    }
    std::printf("]\n}\n");
}

static void print_mesh()
{
    DelaunayMesh mesh(3);
    const double h = 1.0;
    mesh.createBccGrid(Vector3(-2, -2, -2), Vector3(2, 2, 2), h);
    std::printf("{\n  \"source\": \"jukan_koodit/Mesh/DelaunayMesh.cpp:178-219, Mesh.cpp:1479-1512\",\n");
    std::printf("  \"h\": %.17g,\n", h);
    // Interior nodes: the corner node at the origin and the body-centre node at (0.5,0.5,0.5).
    const Vector4 want[2] = {Vector4(0, 0, 0, 0), Vector4(0.5, 0.5, 0.5, 0)};
    std::printf("  \"nodes\": [");
    for (int w = 0; w < 2; w++) {
        uint best = 0;
        double bd = 1e30;
        for (uint n = 0; n < mesh.getNodeSize(); n++) {
            const double d = (mesh.getNodePosition(n) - want[w]).lensq();
            if (d < bd) { bd = d; best = n; }
        }
        const Vector4 p = mesh.getNodePosition(best);
        const double nh = mesh.getNodeHodge(best);
        std::printf("%s\n    {\"position\": [%.17g, %.17g, %.17g], \"node_hodge\": %.17g, \"edges\": [",
                    w ? "," : "", p.x, p.y, p.z, nh);
        const Buffer<uint> &e = mesh.getNodeEdges(best);
        for (uint k = 0; k < e.size(); k++) {
            const uint o = mesh.getEdgeOtherNode(e[k], best);
            const Vector4 q = mesh.getNodePosition(o) - p;
            std::printf("%s[%.17g, %.17g, %.17g, %.17g]", k ? ", " : "", q.x, q.y, q.z,
                        mesh.getEdgeHodge(e[k]) / nh);
        }
        std::printf("]}");
    }
    std::printf("\n  ],\n");
    // Interior bodies (tetrahedra) near the centre: circumcentre, 1/volume, and
    // the Laplacian weight getBodyHodge/getFaceHodge across each face.
    std::printf("  \"bodies\": [");
    int printed = 0;
    for (uint b = 0; b < mesh.getBodySize() && printed < 12; b++) {
        const Vector4 c = mesh.getBodyPosition(b);
        if (std::fabs(c.x) > 0.6 || std::fabs(c.y) > 0.6 || std::fabs(c.z) > 0.6) continue;
        const Buffer<uint> &f = mesh.getBodyFaces(b);
        std::printf("%s\n    {\"position\": [%.17g, %.17g, %.17g], \"body_hodge\": %.17g, \"faces\": [",
                    printed ? "," : "", c.x, c.y, c.z, mesh.getBodyHodge(b));
        for (uint k = 0; k < f.size(); k++) {
            const Buffer<uint> &fb = mesh.getFaceBodies(f[k]);
            uint other = (fb[0] == b) ? (fb.size() > 1 ? fb[1] : NONE) : fb[0];
            Vector4 q(0, 0, 0, 0);
            if (other != NONE) q = mesh.getBodyPosition(other) - c;
            std::printf("%s[%.17g, %.17g, %.17g, %.17g]", k ? ", " : "", q.x, q.y, q.z,
                        mesh.getBodyHodge(b) / mesh.getFaceHodge(f[k]));
        }
        std::printf("]}");
        printed++;
    }
    std::printf("\n  ]\n}\n");
}

static void print_vortex(const char *path)
{
    VortexState state;
    if (!state.load(path)) { std::fprintf(stderr, "cannot load %s\n", path); std::exit(2); }
    const ddouble eps = 1e-5 * state.searchFunctionMax();
    const ddouble maxr = state.searchMaxR(eps);
    const ddouble maxz = state.searchMaxZ(eps);
    const ddouble curv = state.integrateCurvature();
    const ddouble block_scale = PIx2 / (20.0 * std::sqrt(curv));
    std::printf("{\n  \"source\": \"koodit/GrossPitaevskii/VortexState.cpp, GPUGrossPitaevskii_BCC.cu:503-548\",\n");
    std::printf("  \"kappa\": %u, \"g\": %.17g, \"mu\": %.17g,\n", state.getKappa(), state.getG(), state.getMu());
    std::printf("  \"function_max\": %.17g, \"maxr\": %.17g, \"maxz\": %.17g,\n", state.searchFunctionMax(), maxr, maxz);
    std::printf("  \"curvature\": %.17g, \"block_scale\": %.17g,\n", curv, block_scale);
    std::printf("  \"min_r\": %.17g, \"max_r\": %.17g, \"max_z\": %.17g,\n", state.getMinR(), state.getMaxR(), state.getMaxZ());
    // psi at a deterministic set of points
    std::printf("  \"psi_samples\": [");
    Random pr(7);
    for (int i = 0; i < 64; i++) {
        Vector3 p(20.0 * (pr.getUniform() - 0.5), 20.0 * (pr.getUniform() - 0.5), 70.0 * (pr.getUniform() - 0.5));
        if (i == 0) p = Vector3(0, 0, 0);
        if (i == 1) p = Vector3(1e-31, 0, 0);
        if (i == 2) p = Vector3(3.0, 4.0, 35.0);
        const Complex c = state.getPsi(p);
        std::printf("%s[%.17g, %.17g, %.17g, %.17g, %.17g]", i ? ", " : "", p.x, p.y, p.z, c.r, c.i);
    }
    std::printf("],\n  \"phase_samples\": [");
    const double times[4] = {-0.5e-3, -0.5 * 0.000123, 0.0, 1.25};
    for (int i = 0; i < 4; i++) {
        const Complex c = state.getPhase(times[i]);
        std::printf("%s[%.17g, %.17g, %.17g]", i ? ", " : "", times[i], c.r, c.i);
    }
    std::printf("],\n  \"potential_v3_samples\": [");
    for (int i = 0; i < 4; i++) {
        const Vector3 p(0.5 * i - 1.0, 0.25 * i, 3.0 * i - 2.0);
        std::printf("%s[%.17g, %.17g, %.17g, %.17g]", i ? ", " : "", p.x, p.y, p.z, potentialV3(p));
    }
    std::printf("],\n  \"uniform_circle_seed54363\": [");
    Random rnd(54363);
    for (int i = 0; i < 256; i++) {
        const Vector2 c = rnd.getUniformCircle();
        std::printf("%s[%.17g, %.17g]", i ? ", " : "", c.x, c.y);
    }
    std::printf("],\n  \"uint_seed54363\": [");
    Random rnd2(54363);
    for (int i = 0; i < 16; i++) std::printf("%s%u", i ? ", " : "", rnd2.getUint());
    std::printf("]\n}\n");
}

// Restates the host set-up of integrateInTime (GPUGrossPitaevskii_BCC.cu:222-348)
// over the reference's own functions, for a caller-chosen block_scale.
static void run_setup(const char *state_path, double block_scale, const char *out_bin)
{
    VortexState state;
    if (!state.load(state_path)) { std::fprintf(stderr, "cannot load %s\n", state_path); std::exit(2); }
    const ddouble eps = 1e-5 * state.searchFunctionMax();
    const ddouble maxr = state.searchMaxR(eps);
    const ddouble maxz = state.searchMaxZ(eps);
    const Vector3 minp(-maxr, -maxr, -maxz), maxp(maxr, maxr, maxz);
    const Vector3 domain = maxp - minp;
    const uint xsize = uint(domain.x / (block_scale * BLOCK_WIDTH.x)) + 1;
    const uint ysize = uint(domain.y / (block_scale * BLOCK_WIDTH.y)) + 1;
    const uint zsize = uint(domain.z / (block_scale * BLOCK_WIDTH.z)) + 1;
    const Vector3 p0 = 0.5 * (minp + maxp - block_scale * Vector3(BLOCK_WIDTH.x * xsize, BLOCK_WIDTH.y * ysize, BLOCK_WIDTH.z * zsize));
    Buffer<Vector3> bpos;
    getPositions(bpos);
    const uint bsize = bpos.size();
    const size_t n = size_t(xsize) * ysize * zsize * bsize;
    std::vector<double> psi0(2 * n), pot(n), even(2 * n), odd(2 * n);
    ddouble g = state.getG();
    ddouble maxpot = 0.0;
    for (uint k = 0; k < zsize; k++)
        for (uint j = 0; j < ysize; j++)
            for (uint i = 0; i < xsize; i++)
                for (uint l = 0; l < bsize; l++) {
                    const size_t ii = ((size_t(k) * ysize + j) * xsize + i) * bsize + l;
                    const Vector3 p(p0.x + block_scale * (i * BLOCK_WIDTH.x + bpos[l].x),
                                    p0.y + block_scale * (j * BLOCK_WIDTH.y + bpos[l].y),
                                    p0.z + block_scale * (k * BLOCK_WIDTH.z + bpos[l].z));
                    const Complex c = state.getPsi(p);
                    psi0[2 * ii] = c.r;
                    psi0[2 * ii + 1] = c.i;
                    pot[ii] = potentialV3(p);
                    const ddouble poti = pot[ii] + g * c.normsq();
                    if (poti > maxpot) maxpot = poti;
                }
    Buffer<int2> lapind;
    ddouble lapfac = -0.5 * getLaplacian(lapind, 1, 8, 64) / (block_scale * block_scale);
    const uint lapsize = lapind.size() / bsize;
    ddouble lapfac0 = lapsize * (-lapfac);
    const double iteration_period = 1.0;
    const uint steps_per_iteration = uint(iteration_period * (maxpot + lapfac0)) + 1;
    const ddouble dt = iteration_period / ddouble(steps_per_iteration);
    g *= dt;
    lapfac *= dt;
    lapfac0 *= dt;
    for (size_t i = 0; i < n; i++) pot[i] *= dt;
    const Complex oddPhase = state.getPhase(-0.5 * dt);
    Random rnd(54363);
    for (uint k = 0; k < zsize; k++)
        for (uint j = 0; j < ysize; j++)
            for (uint i = 0; i < xsize; i++)
                for (uint l = 0; l < bsize; l++) {
                    const size_t ii = ((size_t(k) * ysize + j) * xsize + i) * bsize + l;
                    const Vector2 c = 0.01 * rnd.getUniformCircle();
                    const Complex noise(c.x + 1.0, c.y);
                    const Complex noised = Complex(psi0[2 * ii], psi0[2 * ii + 1]) * noise;
                    even[2 * ii] = noised.r;
                    even[2 * ii + 1] = noised.i;
                    odd[2 * ii] = oddPhase.r * noised.r - oddPhase.i * noised.i;
                    odd[2 * ii + 1] = oddPhase.i * noised.r + oddPhase.r * noised.i;
                }
    FILE *f = std::fopen(out_bin, "wb");
    if (!f) { std::fprintf(stderr, "cannot write %s\n", out_bin); std::exit(2); }
    std::fwrite(even.data(), sizeof(double), even.size(), f);
    std::fwrite(odd.data(), sizeof(double), odd.size(), f);
    std::fwrite(pot.data(), sizeof(double), pot.size(), f);
    std::fclose(f);
    std::printf("{\n  \"source\": \"koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:222-348\",\n");
    std::printf("  \"block_scale\": %.17g, \"xsize\": %u, \"ysize\": %u, \"zsize\": %u, \"bsize\": %u,\n",
                block_scale, xsize, ysize, zsize, bsize);
    std::printf("  \"p0\": [%.17g, %.17g, %.17g],\n", p0.x, p0.y, p0.z);
    std::printf("  \"minp\": [%.17g, %.17g, %.17g], \"maxp\": [%.17g, %.17g, %.17g],\n",
                minp.x, minp.y, minp.z, maxp.x, maxp.y, maxp.z);
    std::printf("  \"maxpot\": %.17g, \"steps_per_iteration\": %u, \"dt\": %.17g,\n", maxpot, steps_per_iteration, dt);
    std::printf("  \"lapfac_dt\": %.17g, \"lapfac0_dt\": %.17g, \"g_dt\": %.17g,\n", lapfac, lapfac0, g);
    std::printf("  \"odd_phase\": [%.17g, %.17g],\n", oddPhase.r, oddPhase.i);
    std::printf("  \"layout\": \"float64; even[z][y][x][slot][re,im], then odd (same), then pot*dt[z][y][x][slot]\"\n}\n");
}

// The reference's two debug outputs for the even field of a set-up file written
// by `setup` (block order, interior blocks): the BMP slice of SAVE_PICTURE
// (GPUGrossPitaevskii_BCC.cu:424-441) and the MetaImage volume of SAVE_VOLUME
// (:443-468), both on the padded host array the reference keeps, written by
// the reference's own Picture::save and saveVolumeMap.  The per-pixel loops are
// restated from those lines (they sit inside integrateInTime).
#include "jukan_koodit/Output/Picture.hpp"
bool saveVolumeMap(const std::string &path, const Buffer<ushort> &vol, const uint xsize, const uint ysize,
                   const uint zsize, const Vector3 &h);
static void run_outputs(const char *setup_bin, uint xsize, uint ysize, uint zsize, double block_scale, double fmax,
                        const char *bmp, const char *mhd)
{
    const size_t n = size_t(xsize) * ysize * zsize * 12;
    std::vector<double> even(2 * n);
    FILE *f = std::fopen(setup_bin, "rb");
    if (!f || std::fread(even.data(), sizeof(double), even.size(), f) != even.size()) { std::fprintf(stderr, "bad %s\n", setup_bin); std::exit(2); }
    std::fclose(f);
    const uint dxsize = xsize + 2, dysize = ysize + 2, dzsize = zsize + 2, bsize = 12;
    // padded host array h_evenPsi[(k*dysize + j)*dxsize + i].values[l]
    std::vector<double> h(size_t(dxsize) * dysize * dzsize * 24, 0.0);
    for (uint k = 0; k < zsize; k++)
        for (uint j = 0; j < ysize; j++)
            for (uint i = 0; i < xsize; i++)
                for (uint l = 0; l < 12; l++) {
                    const size_t src = ((size_t(k) * ysize + j) * xsize + i) * 12 + l;
                    const size_t dst = ((size_t(k + 1) * dysize + (j + 1)) * dxsize + (i + 1)) * 24 + 2 * l;
                    h[dst] = even[2 * src];
                    h[dst + 1] = even[2 * src + 1];
                }
    // picture (:426-440)
    Picture pic(dxsize, dysize);
    const uint kk = zsize / 2 + 1;
    for (uint j = 0; j < dysize; j++)
        for (uint i = 0; i < dxsize; i++) {
            const size_t idx = size_t(kk) * dxsize * dysize + j * dxsize + i;
            const double x = h[idx * 24], y = h[idx * 24 + 1];
            const double norm = sqrt(x * x + y * y);
            pic.setColor(i, j, 5.0 * Vector4(x, norm, y, 1.0));
        }
    pic.save(bmp, false);
    // volume (:445-467), including the reference's sum over values[0]
    const ddouble unit = 60000.0 / (bsize * fmax * fmax);
    Buffer<ushort> vol(dxsize * dysize * dzsize);
    for (uint k = 0; k < dzsize; k++)
        for (uint j = 0; j < dysize; j++)
            for (uint i = 0; i < dxsize; i++) {
                const size_t idx = size_t(k) * dxsize * dysize + j * dxsize + i;
                ddouble sum = 0.0;
                for (uint l = 0; l < bsize; l++) sum += h[idx * 24] * h[idx * 24] + h[idx * 24 + 1] * h[idx * 24 + 1];
                sum *= unit;
                vol[idx] = (sum > 65535.0 ? 65535 : ushort(sum));
            }
    saveVolumeMap(mhd, vol, dxsize, dysize, dzsize, block_scale * BLOCK_WIDTH);
    std::printf("{\"unit\": %.17g, \"slice_k\": %u, \"dims\": [%u, %u, %u]}\n", unit, kk, dxsize, dysize, dzsize);
}

// A small vortex state made by the reference's own axisymmetric relaxation
// (VortexState::setRange + iterateSolution, VortexState.cpp:42-47,109-196; the
// potential is the reference's potentialRZ, GPUGrossPitaevskii_BCC.cu:28-31).
extern ddouble potentialRZ(const ddouble r, const ddouble z);
static void make_state(const char *out, uint kappa, double g, double rstep, uint iters)
{
    VortexState state;
    state.setKappa(kappa);
    state.setG(g);
    state.setRange(0.0, 15.0, 35.0, rstep, rstep);
    state.iterateSolution(potentialRZ, iters, 1e-29);
    if (!state.save(out)) { std::fprintf(stderr, "cannot write %s\n", out); std::exit(2); }
    std::printf("{\"kappa\": %u, \"g\": %.17g, \"mu\": %.17g, \"rstep\": %.17g, \"iterations\": %u}\n", kappa, g,
                state.getMu(), rstep, iters);
}

int main(int argc, char **argv)
{
    if (argc < 2) { std::fprintf(stderr, "usage: %s tables|mesh|vortex STATE|setup STATE BS OUT|makestate OUT\n", argv[0]); return 2; }
    const std::string cmd = argv[1];
    if (cmd == "tables") print_tables();
    else if (cmd == "mesh") print_mesh();
    else if (cmd == "vortex" && argc >= 3) print_vortex(argv[2]);
    else if (cmd == "setup" && argc >= 5) run_setup(argv[2], std::atof(argv[3]), argv[4]);
    else if (cmd == "makestate" && argc >= 3) make_state(argv[2], 20, 5000.0, 0.25, 3000);
    else if (cmd == "outputs" && argc >= 10)
        run_outputs(argv[2], std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]), std::atof(argv[6]),
                    std::atof(argv[7]), argv[8], argv[9]);
    else { std::fprintf(stderr, "bad arguments\n"); return 2; }
    return 0;
}
