// Host side of the octree build: mesh input and the level sets, bit-exact with the
// reference's octree.c.  The interaction lists are built on the GPU (octree_gpu.cu).
#pragma once
#include <vector>
#include <string>

namespace fmm {

struct HostTree {
    int lmin = 2, lmax = 0;
    double d = 0.0;
    double pt_min[3] = {0, 0, 0};
    std::vector<std::vector<long long>> sets; // sets[l] for l = lmin..lmax, reference order
    std::vector<long long> elem_key;          // leaf Morton key per element (double centroid)
    std::vector<int> elem_leaf;               // index into sets[lmax] per element
};

// readOBJ/findNum (octree.c:563-619): 48-character fgets chunks, 'v' and 'f' lines.
int read_obj(const char *path, std::vector<double> &V, std::vector<int> &F);

// triCentroid_d (structs.cu:126-131)
void centroid(const double *n0, const double *n1, const double *n2, double *c);

// findBoundingCube (octree.c:681-747) including the z seeding from y (kept for parity)
void bounding_cube(const std::vector<double> &P, double eps, double *pt_min, double *d);

// pnt2boxnum (octree.c:158-183) on a scaled point
long long morton_key(const double *s, int l);

// deterLmax (octree.c:635-679); 11 on a tie as in the reference
int deter_lmax(const std::vector<double> &S, int s);

// createSet (octree.c:393-410): unique values in order of first occurrence
std::vector<long long> first_occurrence(const std::vector<long long> &v);

// srcBoxes + FMMLevelSet (octree.c:749-768, 890-906); depth > 0 overrides deterLmax
int build_tree(const std::vector<double> &V, const std::vector<int> &F, int s, int depth, HostTree &T);

// box integer coordinates and number at level l (bitIntleave/bitDeintleave)
void box_xyz(long long num, int l, int *x, int *y, int *z);
long long box_num(int x, int y, int z, int l);

} // namespace fmm
