// gpe_lattice.cpp - DEC stencil tables of the two BCC discretisations, derived
// from the geometry of the body-centred-cubic Delaunay tetrahedralisation.
//
// Both discretisations live on the same mesh: lattice points at the cube corners
// and cube centres (two interpenetrating simple-cubic sublattices), and the
// Delaunay tetrahedra between them (12 per cube, all congruent).
//
//  * TETRA12 - the reference's discretisation (koodit/GrossPitaevskii/
//    GPUGrossPitaevskii_BCC.cu:69-142): one value per tetrahedron, stored at its
//    circumcentre; 12 values per cubic block; 4 neighbours (one across each
//    face).  Weight = getBodyHodge/getFaceHodge of the reference Mesh library
//    (jukan_koodit/Mesh/Mesh.cpp:1479-1512) = |face| / (|tet| * |dual edge|).
//    Lengths are in units of block_scale with the block edge sqrt(8) (:70).
//  * BCC2 - one value per lattice point (corner + centre, 2 per block); 14
//    neighbours (8 body diagonals, 6 axial).  Weight = getEdgeHodge/getNodeHodge
//    = |dual face| / (|edge| * |dual cell|).  Lengths in units of the cube edge.
//
// Everything is computed here from integer coordinates in units of 1/8 of the
// block edge; nothing is tabulated except the order in which the reference
// numbers the 12 circumcentres of a block (its storage format, :73-89).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <vector>

#include "gpe_internal.h"

namespace gpe {
namespace {

using I3 = std::array<int, 3>;

I3 add(const I3 &a, const I3 &b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
I3 sub(const I3 &a, const I3 &b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
long dist2(const I3 &a, const I3 &b)
{
    long s = 0;
    for (int k = 0; k < 3; k++) s += long(a[k] - b[k]) * (a[k] - b[k]);
    return s;
}
int floordiv8(int v) { return (v >= 0) ? v / 8 : -((-v + 7) / 8); }

struct V3 {
    double x, y, z;
};
V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double norm(V3 a) { return std::sqrt(dot(a, a)); }
V3 tov(const I3 &a) { return {double(a[0]), double(a[1]), double(a[2])}; }

// A BCC lattice whose corner sublattice sits at offset `o` (in 1/8 block units)
// inside each block; the centre sublattice is at o + (4,4,4).
struct Bcc {
    I3 o;
    // Lattice points within a cube of +-R blocks around the origin block.
    std::vector<I3> points(int R) const
    {
        std::vector<I3> p;
        for (int sub = 0; sub < 2; sub++)
            for (int i = -R; i <= R; i++)
                for (int j = -R; j <= R; j++)
                    for (int k = -R; k <= R; k++)
                        p.push_back({o[0] + 4 * sub + 8 * i, o[1] + 4 * sub + 8 * j, o[2] + 4 * sub + 8 * k});
        return p;
    }
    // The 12 Delaunay circumcentres around a corner point: one coordinate +4,
    // one +-2, one 0 (relative to the corner point; the tetragonal disphenoids
    // of the BCC lattice).  Returned modulo the block, i.e. in [0,8)^3.
    std::vector<I3> circumcentres_in_block() const
    {
        std::vector<I3> c;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                if (b == a) continue;
                for (int sgn = -1; sgn <= 1; sgn += 2) {
                    I3 v = {0, 0, 0};
                    v[a] = 4;
                    v[b] = 2 * sgn;
                    I3 p = add(o, v);
                    for (int k = 0; k < 3; k++) p[k] = ((p[k] % 8) + 8) % 8;
                    c.push_back(p);
                }
            }
        return c;
    }
};

// The four lattice points nearest to a circumcentre are the tetrahedron's vertices.
std::array<I3, 4> tet_vertices(const std::vector<I3> &pts, const I3 &c)
{
    std::vector<std::pair<long, I3>> d;
    d.reserve(pts.size());
    for (const I3 &p : pts) d.push_back({dist2(p, c), p});
    std::partial_sort(d.begin(), d.begin() + 5, d.end(),
                      [](const std::pair<long, I3> &a, const std::pair<long, I3> &b) { return a.first < b.first; });
    std::array<I3, 4> v;
    for (int k = 0; k < 4; k++) v[k] = d[k].second;
    std::sort(v.begin(), v.end());
    return v;
}

double tet_volume(const std::array<I3, 4> &v)
{
    V3 a = vsub(tov(v[1]), tov(v[0])), b = vsub(tov(v[2]), tov(v[0])), c = vsub(tov(v[3]), tov(v[0]));
    return std::fabs(dot(a, cross(b, c))) / 6.0;
}

struct Entry {
    int dx, dy, dz, slot;
    double w;
};

// The weights and volumes of these lattices are small dyadic rationals (1.5,
// 0.75, 0.25, 0.5) or irrational (sqrt(32/9)); computed from the geometry they
// carry a few ulp of rounding.  A value within 8 ulp of a multiple of 2^-32 is
// taken to be that multiple, so that the factors built from it are the ones the
// reference builds from its exact constants (getLaplacian returns 1.5).
double snap_dyadic(double v)
{
    const double r = std::ldexp(std::nearbyint(std::ldexp(v, 32)), -32);
    const double ulp = std::nextafter(std::fabs(v), INFINITY) - std::fabs(v);
    return std::fabs(r - v) <= 8.0 * ulp ? r : v;
}

void finish(gpe_lattice_info *info, std::vector<std::vector<Entry>> &tab)
{
    // Weight classes: distinct weights, largest first.
    std::vector<double> cls;
    for (auto &row : tab)
        for (auto &e : row) {
            bool found = false;
            for (double c : cls)
                if (std::fabs(c - e.w) <= 1e-12 * std::fabs(c)) found = true;
            if (!found) cls.push_back(snap_dyadic(e.w));
        }
    std::sort(cls.begin(), cls.end(), std::greater<double>());
    info->classes = int(cls.size());
    for (size_t c = 0; c < cls.size() && c < 2; c++) info->class_weight[c] = cls[c];
    for (size_t s = 0; s < tab.size(); s++) {
        auto &row = tab[s];
        auto cls_of = [&](const Entry &e) {
            for (size_t c = 0; c < cls.size(); c++)
                if (std::fabs(cls[c] - e.w) <= 1e-12 * std::fabs(cls[c])) return int(c);
            return -1;
        };
        // Summation order: by weight class, then (dz, dy, dx, slot).
        std::sort(row.begin(), row.end(), [&](const Entry &a, const Entry &b) {
            int ca = cls_of(a), cb = cls_of(b);
            if (ca != cb) return ca < cb;
            if (a.dz != b.dz) return a.dz < b.dz;
            if (a.dy != b.dy) return a.dy < b.dy;
            if (a.dx != b.dx) return a.dx < b.dx;
            return a.slot < b.slot;
        });
        for (size_t k = 0; k < row.size(); k++) {
            info->entry[s][k][0] = row[k].dx;
            info->entry[s][k][1] = row[k].dy;
            info->entry[s][k][2] = row[k].dz;
            info->entry[s][k][3] = row[k].slot;
            info->entry[s][k][4] = cls_of(row[k]);
        }
    }
}

// The reference numbers a block's 12 circumcentres in this order (block-relative,
// units of 1/8 block edge; GPUGrossPitaevskii_BCC.cu:77-88 stores them scaled by
// 1/sqrt(8) of a sqrt(8)-wide block).  Values are stored per block in this order.
const int kTetraSlotOrder[12][3] = {{1, 3, 7}, {7, 1, 3}, {7, 3, 1}, {7, 3, 5}, {7, 5, 3}, {1, 7, 3},
                                    {3, 7, 1}, {3, 7, 5}, {5, 7, 3}, {3, 1, 7}, {3, 5, 7}, {5, 3, 7}};

gpe_status build_tetra12(gpe_lattice_info *info)
{
    // The reference's circumcentres belong to a lattice whose corner points sit
    // at (3,3,3)/8 of the block.
    Bcc bcc{{3, 3, 3}};
    const std::vector<I3> pts = bcc.points(2);
    std::vector<I3> cc = bcc.circumcentres_in_block();
    std::vector<I3> order(12);
    for (int s = 0; s < 12; s++) order[s] = {kTetraSlotOrder[s][0], kTetraSlotOrder[s][1], kTetraSlotOrder[s][2]};
    // The geometric set and the storage order must describe the same 12 points.
    {
        std::set<I3> a(cc.begin(), cc.end()), b(order.begin(), order.end());
        if (a != b) return GPE_ERR_INTERNAL;
    }
    // All circumcentres of the 27 surrounding blocks, keyed by vertex set.
    std::map<std::array<I3, 4>, std::array<int, 4>> owner;  // -> (dx,dy,dz,slot)
    std::map<std::array<I3, 4>, I3> centre;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++)
                for (int s = 0; s < 12; s++) {
                    I3 c = add(order[s], {8 * dx, 8 * dy, 8 * dz});
                    auto v = tet_vertices(pts, c);
                    owner[v] = {dx, dy, dz, s};
                    centre[v] = c;
                }
    std::vector<std::vector<Entry>> tab(12);
    double vol = 0.0;
    for (int s = 0; s < 12; s++) {
        auto v = tet_vertices(pts, order[s]);
        vol = tet_volume(v);
        for (int drop = 0; drop < 4; drop++) {
            std::vector<I3> face;
            for (int k = 0; k < 4; k++)
                if (k != drop) face.push_back(v[k]);
            int hits = 0;
            for (auto &kv : owner) {
                if (kv.first == v) continue;
                int shared = 0;
                for (const I3 &p : face)
                    if (std::find(kv.first.begin(), kv.first.end(), p) != kv.first.end()) shared++;
                if (shared != 3) continue;
                hits++;
                const V3 a = tov(face[0]), b = tov(face[1]), c = tov(face[2]);
                const double area = 0.5 * norm(cross(vsub(b, a), vsub(c, a)));
                const double dual = norm(vsub(tov(centre[kv.first]), tov(order[s])));
                // In 1/8-block units; block edge = sqrt(8) block_scale, so one
                // unit is sqrt(8)/8 block_scale and 1/unit^2 = 8 / block_scale^2.
                const double w = area / (tet_volume(v) * dual) * 8.0;
                tab[s].push_back({kv.second[0], kv.second[1], kv.second[2], kv.second[3], w});
            }
            if (hits != 1) return GPE_ERR_INTERNAL;
        }
    }
    info->slots = 12;
    info->neighbours = 4;
    info->block_width = std::sqrt(8.0);
    // tetrahedron volume: vol units of (sqrt(8)/8)^3 block_scale^3
    info->cell_volume = vol * std::pow(std::sqrt(8.0) / 8.0, 3);
    // position = (eighths of the block) * block edge / 8, rounded as the reference
    // rounds it: (1/sqrt(8)) * eighths (GPUGrossPitaevskii_BCC.cu:75-88), so the
    // doubles equal its getPositions output
    const double inv_sqrt8 = 1.0 / std::sqrt(8.0);
    for (int s = 0; s < 12; s++)
        for (int k = 0; k < 3; k++) info->position[s][k] = inv_sqrt8 * double(order[s][k]);
    finish(info, tab);
    // Summation order of the four neighbours: the order in which the reference's
    // getLaplacian lists them (GPUGrossPitaevskii_BCC.cu:90-142), which its kernel
    // sums in.  In geometric terms: a circumcentre has one coordinate at 7/8 of the
    // block (its major axis).  First come the two neighbours whose displacement has
    // no component along that axis, then the other two.  Within each pair the two
    // displacements differ in one component; the first pair is ordered by it
    // ascending, the second descending.
    for (int s = 0; s < 12; s++) {
        int m = 0;
        for (int k = 1; k < 3; k++)
            if (order[s][k] > order[s][m]) m = k;
        std::array<std::array<int, 5>, 4> row;
        std::array<I3, 4> disp;
        for (int k = 0; k < 4; k++) {
            for (int c = 0; c < 5; c++) row[k][c] = info->entry[s][k][c];
            const I3 &to = order[row[k][3]];
            disp[k] = {8 * row[k][0] + to[0] - order[s][0], 8 * row[k][1] + to[1] - order[s][1],
                       8 * row[k][2] + to[2] - order[s][2]};
        }
        std::array<int, 4> idx = {0, 1, 2, 3};
        std::vector<int> flat, axial;
        for (int k : idx) (disp[k][m] == 0 ? flat : axial).push_back(k);
        if (flat.size() != 2 || axial.size() != 2) return GPE_ERR_INTERNAL;
        auto order_pair = [&](std::vector<int> &pair, bool ascending) {
            const I3 &a = disp[pair[0]], &b = disp[pair[1]];
            int c = 0;
            while (c < 3 && a[c] == b[c]) c++;
            if (c == 3) return false;
            if ((a[c] < b[c]) != ascending) std::swap(pair[0], pair[1]);
            return true;
        };
        if (!order_pair(flat, true) || !order_pair(axial, false)) return GPE_ERR_INTERNAL;
        const int seq[4] = {flat[0], flat[1], axial[0], axial[1]};
        for (int k = 0; k < 4; k++)
            for (int c = 0; c < 5; c++) info->entry[s][k][c] = row[seq[k]][c];
    }
    return GPE_OK;
}

gpe_status build_bcc2(gpe_lattice_info *info)
{
    // Corner sublattice at (1/4,1/4,1/4) of the block, centre sublattice at
    // (3/4,3/4,3/4): the value cloud of a block grid is then symmetric under
    // inversion through the grid centre.
    Bcc bcc{{2, 2, 2}};
    const std::vector<I3> pts = bcc.points(2);
    const I3 slot_pos[2] = {{2, 2, 2}, {6, 6, 6}};
    // All tetrahedra touching the two slot points: circumcentres of the 27
    // surrounding blocks.
    std::vector<std::pair<std::array<I3, 4>, I3>> tets;
    std::vector<I3> cc = bcc.circumcentres_in_block();
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++)
                for (const I3 &c0 : cc) {
                    I3 c = add(c0, {8 * dx, 8 * dy, 8 * dz});
                    tets.push_back({tet_vertices(pts, c), c});
                }
    std::vector<std::vector<Entry>> tab(2);
    double dual_volume = 0.0;
    for (int s = 0; s < 2; s++) {
        const I3 n = slot_pos[s];
        // Edges of n: other vertices of the tetrahedra containing n.
        std::set<I3> nbrs;
        for (auto &t : tets)
            if (std::find(t.first.begin(), t.first.end(), n) != t.first.end())
                for (const I3 &p : t.first)
                    if (p != n) nbrs.insert(p);
        double vol = 0.0;
        for (const I3 &m : nbrs) {
            // Dual face of edge (n,m): circumcentres of the tetrahedra sharing it,
            // ordered by angle around the edge; area by a fan from their centroid.
            std::vector<V3> ring;
            for (auto &t : tets) {
                bool hn = std::find(t.first.begin(), t.first.end(), n) != t.first.end();
                bool hm = std::find(t.first.begin(), t.first.end(), m) != t.first.end();
                if (hn && hm) ring.push_back(tov(t.second));
            }
            if (ring.size() < 3) return GPE_ERR_INTERNAL;
            const V3 e = vsub(tov(m), tov(n));
            const double elen = norm(e);
            V3 cen{0, 0, 0};
            for (auto &p : ring) cen = {cen.x + p.x, cen.y + p.y, cen.z + p.z};
            cen = {cen.x / ring.size(), cen.y / ring.size(), cen.z / ring.size()};
            V3 u = vsub(ring[0], cen);
            V3 w = cross(e, u);
            std::sort(ring.begin(), ring.end(), [&](const V3 &a, const V3 &b) {
                V3 ra = vsub(a, cen), rb = vsub(b, cen);
                return std::atan2(dot(ra, w), dot(ra, u)) < std::atan2(dot(rb, w), dot(rb, u));
            });
            double area = 0.0;
            for (size_t k = 0; k < ring.size(); k++) {
                V3 a = vsub(ring[k], cen), b = vsub(ring[(k + 1) % ring.size()], cen);
                area += 0.5 * norm(cross(a, b));
            }
            vol += (0.5 * elen) * area / 3.0;  // pyramid over the dual face
            const I3 d = sub(m, {0, 0, 0});
            const int bx = floordiv8(d[0]), by = floordiv8(d[1]), bz = floordiv8(d[2]);
            const I3 inblock = {d[0] - 8 * bx, d[1] - 8 * by, d[2] - 8 * bz};
            int slot = (inblock == slot_pos[0]) ? 0 : (inblock == slot_pos[1] ? 1 : -1);
            if (slot < 0) return GPE_ERR_INTERNAL;
            tab[s].push_back({bx, by, bz, slot, area / elen});  // divided by the dual volume below
        }
        for (auto &en : tab[s]) en.w /= vol;
        // Units: 1/8 block edge; weights scale as 1/length^2 -> x 64 / a^2.
        for (auto &en : tab[s]) en.w *= 64.0;
        dual_volume = vol / 512.0;
        if (tab[s].size() != 14) return GPE_ERR_INTERNAL;
    }
    info->slots = 2;
    info->neighbours = 14;
    info->block_width = 1.0;
    info->cell_volume = snap_dyadic(dual_volume);
    for (int s = 0; s < 2; s++)
        for (int k = 0; k < 3; k++) info->position[s][k] = slot_pos[s][k] / 8.0;
    finish(info, tab);
    return GPE_OK;
}

}  // namespace

gpe_status build_lattice(gpe_lattice lattice, gpe_lattice_info *info)
{
    std::memset(info, 0, sizeof(*info));
    info->lattice = lattice;
    if (lattice == GPE_LATTICE_TETRA12) return build_tetra12(info);
    if (lattice == GPE_LATTICE_BCC2) return build_bcc2(info);
    return GPE_ERR_INVALID_ARGUMENT;
}

}  // namespace gpe
