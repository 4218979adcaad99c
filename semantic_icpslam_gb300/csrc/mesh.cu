// Marching-cubes mesher of the voxel-block map.
//
// Reference: MeshEngine (Mapping/MeshScene.cu:4-297: readVertexAndColor,
// readNormal, interp, buildVertexList, MarchingCube) and MeshScene (:307-
// 356), driven by Mapping::CreateModel (Mapping/Mapping.cc:183-192).
//
// GB300 form: the allocated-entry index replaces CheckBlockKernel's scan of
// every hash entry; one 64-thread CTA per block (one thread per (x, y) cube
// column, z looped, as the reference's (8, 8) launch), a per-thread cache
// of the last block looked up, and the output triangles appended with one
// atomic per cube.  The tables are built at compile time by the rule below
// instead of being carried as data.
#include "sf_kernels.cuh"

namespace sf {
namespace {

// Cube corners 0..7 at (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1)
// (1,1,1) (0,1,1) and edges 0..11 between corners (0,1) (1,2) (2,3) (3,0)
// (4,5) (5,6) (6,7) (7,4) (0,4) (1,5) (2,6) (3,7): MeshScene.cu's
// numbering (readVertexAndColor :117-141, buildVertexList :172-247).
constexpr int kEdgeA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
constexpr int kEdgeB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
// Faces as corner cycles, counterclockwise seen from outside the cube.
constexpr int kFace[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 7, 6, 2}, {0, 4, 7, 3}, {1, 2, 6, 5}};

// The triangle, vertex-count and edge tables.  For a configuration (bit i:
// corner i inside, sdf < 0), every face contributes the segments that cut
// off each of its inside corners -- one segment per inside corner, or one
// per run of inside corners, so a face with two diagonal inside corners
// gets two -- oriented with the inside on the left going counterclockwise.
// The segments chain into closed polygons, each a fan of triangles from its
// lowest-numbered edge.  These polygons are, configuration for
// configuration, those of the classic table MeshScene uses (outline and
// orientation, checked against Mapping/Constant.h); only the split of
// polygons of four or more vertices into triangles is this rule's own.
struct McTables {
  int tri[256][16];  // edge triples, -1 terminated
  int nverts[256];   // 3 x triangles
  int edges[256];    // bit e: edge e crosses the surface
};

constexpr int edge_between(int a, int b) {
  for (int e = 0; e < 12; ++e)
    if ((kEdgeA[e] == a && kEdgeB[e] == b) || (kEdgeA[e] == b && kEdgeB[e] == a)) return e;
  return -1;
}

constexpr McTables build_mc_tables() {
  McTables t{};
  for (int ci = 0; ci < 256; ++ci) {
    int next[12] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
    int edges = 0;
    for (int f = 0; f < 6; ++f) {
      // crossings in counterclockwise order: edge and whether it leaves an
      // inside corner
      int ce[4] = {0, 0, 0, 0}, cin[4] = {0, 0, 0, 0}, n = 0;
      for (int k = 0; k < 4; ++k) {
        const int a = kFace[f][k], b = kFace[f][(k + 1) & 3];
        const int ia = (ci >> a) & 1, ib = (ci >> b) & 1;
        if (ia != ib) {
          ce[n] = edge_between(a, b);
          cin[n] = ia;
          ++n;
        }
      }
      // a crossing into an inside corner pairs with the next crossing out
      // of it: the segment runs from that exit to this entry
      for (int j = 0; j < n; ++j)
        if (cin[j] == 0) {
          const int out = ce[(j + 1) % n];
          next[out] = ce[j];
        }
      for (int j = 0; j < n; ++j) edges |= 1 << ce[j];
    }
    t.edges[ci] = edges;
    int used = 0, ntri = 0;
    for (int k = 0; k < 16; ++k) t.tri[ci][k] = -1;
    for (int start = 0; start < 12; ++start) {
      if (next[start] < 0 || ((used >> start) & 1)) continue;
      // the loop through `start`, the lowest edge of its polygon (edges
      // are visited in increasing order, and a loop is used up whole)
      int loop[12] = {}, len = 0, e = start;
      do {
        loop[len++] = e;
        used |= 1 << e;
        e = next[e];
      } while (e != start && len < 12);
      for (int i = 1; i + 1 < len; ++i) {
        t.tri[ci][3 * ntri + 0] = loop[0];
        t.tri[ci][3 * ntri + 1] = loop[i];
        t.tri[ci][3 * ntri + 2] = loop[i + 1];
        ++ntri;
      }
    }
    t.nverts[ci] = 3 * ntri;
  }
  return t;
}

__constant__ McTables c_mc = build_mc_tables();

// MeshEngine's voxel lookups through a one-entry block cache.
struct MeshLookup {
  const DevMap &m;
  i3 bpos;
  int bptr;
  __device__ MeshLookup(const DevMap &map, i3 own, int own_ptr) : m(map), bpos(own), bptr(own_ptr) {}
  // FindVoxel(int3) (DeviceMap.cu:97-103): the voxel, or null for a
  // missing block (whose default Voxel reads sdf NaN, colour 0).
  __device__ __forceinline__ const sf_voxel *find(i3 v) {
    const i3 b = vox2block(v);
    if (b.x != bpos.x || b.y != bpos.y || b.z != bpos.z) {
      bpos = b;
      bptr = find_block(m, b);
    }
    return bptr < 0 ? nullptr : m.voxels + bptr + vox2local(v);
  }
  __device__ __forceinline__ float sdf(i3 v) {
    const sf_voxel *p = find(v);
    return p ? __ldg(&p->sdf) : nanf_bits();
  }
};

// interp (MeshScene.cu:144-152): fabs(x) < 1e-6 in double is
// fabsf(x) <= 1e-6f for a float x.
__device__ __forceinline__ float mc_interp(float v1, float v2) {
  if (fabsf(0.f - v1) <= 1e-6f) return 0.f;
  if (fabsf(0.f - v2) <= 1e-6f) return 1.f;
  if (fabsf(v1 - v2) <= 1e-6f) return 0.f;
  return (0.f - v1) / (v2 - v1);
}

// uchar3 colour + val * (colour difference): the reference's operators
// take val as an int (VectorMath.h:113-115, 219-221, 297-299), so the
// colour is the first corner's unless val is exactly 1.
__device__ __forceinline__ uchar3 mc_color(uchar3 a, uchar3 b, float val) {
  const int s = (int)val;
  uchar3 d;
  d.x = (unsigned char)(unsigned char)(b.x - a.x) * s;
  d.y = (unsigned char)(unsigned char)(b.y - a.y) * s;
  d.z = (unsigned char)(unsigned char)(b.z - a.z) * s;
  uchar3 r;
  r.x = (unsigned char)(a.x + d.x);
  r.y = (unsigned char)(a.y + d.y);
  r.z = (unsigned char)(a.z + d.z);
  return r;
}

constexpr int kMeshThreads = 64;

// MeshEngine::MarchingCube for the blocks of the allocated-entry index.
__global__ void __launch_bounds__(kMeshThreads) k_mesh(DevMap m, float3 *vert, float3 *norm, uchar3 *col,
                                                       uint32_t max_tri, uint32_t *count) {
  const unsigned nblocks = (unsigned)*m.alloc_count;
  const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;
  const float vs = m.c.voxel_size;
  // corner offsets (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1)
  const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (unsigned b = blockIdx.x; b < nblocks; b += gridDim.x) {
    if (__ldcg(count) >= max_tri) return;
    int4 h = entry_head(m.entries + __ldcg(m.alloc_list + b));
    h.w = checked_ptr(m, h.w);
    if (h.w < 0) continue;
    MeshLookup look(m, mk_i3(h.x, h.y, h.z), h.w);
    for (int z = 0; z < 8; ++z) {
      const i3 pos = mk_i3(h.x * 8 + tx, h.y * 8 + ty, h.z * 8 + z);
      // readVertexAndColor (MeshScene.cu:115-141)
      float sdf[8];
      uchar3 c[8];
      bool ok = true;
      for (int k = 0; k < 8 && ok; ++k) {
        const sf_voxel *p = look.find(mk_i3(pos.x + cx[k], pos.y + cy[k], pos.z + cz[k]));
        sdf[k] = p ? __ldg(&p->sdf) : nanf_bits();
        c[k] = p ? make_uchar3(p->color[0], p->color[1], p->color[2]) : make_uchar3(0, 0, 0);
        ok = !(sdf[k] == 1.0f || isnan(sdf[k]));
      }
      if (!ok) continue;
      // readNormal (MeshScene.cu:43-113): central differences at each
      // corner, the three neighbours outside the cube per corner
      f3 nrm[8];
      const int off[8][3][3] = {
          {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}}, {{2, 0, 0}, {1, -1, 0}, {1, 0, -1}},
          {{2, 1, 0}, {1, 2, 0}, {1, 1, -1}},   {{-1, 1, 0}, {0, 2, 0}, {0, 1, -1}},
          {{-1, 0, 1}, {0, -1, 1}, {0, 0, 2}},  {{2, 0, 1}, {1, -1, 1}, {1, 0, 2}},
          {{2, 1, 1}, {1, 2, 1}, {1, 1, 2}},    {{-1, 1, 1}, {0, 2, 1}, {0, 1, 2}}};
      // the in-cube neighbour of corner k along x, y, z (the other end of
      // its central difference) and the sign: + when the outside
      // neighbour is the upper one
      const int nx[8] = {1, 0, 3, 2, 5, 4, 7, 6}, ny[8] = {3, 2, 1, 0, 7, 6, 5, 4}, nz[8] = {4, 5, 6, 7, 0, 1, 2, 3};
      for (int k = 0; k < 8 && ok; ++k) {
        const float v1 = look.sdf(mk_i3(pos.x + off[k][0][0], pos.y + off[k][0][1], pos.z + off[k][0][2]));
        const float v2 = look.sdf(mk_i3(pos.x + off[k][1][0], pos.y + off[k][1][1], pos.z + off[k][1][2]));
        const float v3 = look.sdf(mk_i3(pos.x + off[k][2][0], pos.y + off[k][2][1], pos.z + off[k][2][2]));
        if (isnan(v1) || isnan(v2) || isnan(v3)) {
          ok = false;
          break;
        }
        nrm[k].x = off[k][0][0] > 0 ? v1 - sdf[nx[k]] : sdf[nx[k]] - v1;
        nrm[k].y = off[k][1][1] > 0 ? v2 - sdf[ny[k]] : sdf[ny[k]] - v2;
        nrm[k].z = off[k][2][2] > 0 ? v3 - sdf[nz[k]] : sdf[nz[k]] - v3;
      }
      if (!ok) continue;
      int ci = 0;
      for (int k = 0; k < 8; ++k) ci |= (sdf[k] < 0.f) << k;
      const int emask = c_mc.edges[ci];
      if (emask == 0 || ci == 0) continue;
      // buildVertexList (MeshScene.cu:172-247)
      f3 vl[12], nl[12];
      uchar3 cl[12];
      for (int e = 0; e < 12; ++e) {
        if (!((emask >> e) & 1)) continue;
        const int a = (e < 8) ? e : e - 8, bc = (e < 8) ? ((e & 3) == 3 ? e - 3 : e + 1) : e - 4;
        // edges 0..7 run a -> a + 1 within a face (3 -> 0, 7 -> 4);
        // edges 8..11 run e - 8 -> e - 4
        const float val = mc_interp(sdf[a], sdf[bc]);
        f3 p;
        p.x = (float)pos.x; p.y = (float)pos.y; p.z = (float)pos.z;
        switch (e) {
          case 0: p.x = (float)pos.x + val; break;
          case 1: p.x = (float)pos.x + 1.f; p.y = (float)pos.y + val; break;
          case 2: p.x = (float)pos.x + (1.f - val); p.y = (float)pos.y + 1.f; break;
          case 3: p.y = (float)pos.y + (1.f - val); break;
          case 4: p.x = (float)pos.x + val; p.z = (float)pos.z + 1.f; break;
          case 5: p.x = (float)pos.x + 1.f; p.y = (float)pos.y + val; p.z = (float)pos.z + 1.f; break;
          case 6: p.x = (float)pos.x + (1.f - val); p.y = (float)pos.y + 1.f; p.z = (float)pos.z + 1.f; break;
          case 7: p.y = (float)pos.y + (1.f - val); p.z = (float)pos.z + 1.f; break;
          case 8: p.z = (float)pos.z + val; break;
          case 9: p.x = (float)pos.x + 1.f; p.z = (float)pos.z + val; break;
          case 10: p.x = (float)pos.x + 1.f; p.y = (float)pos.y + 1.f; p.z = (float)pos.z + val; break;
          default: p.y = (float)pos.y + 1.f; p.z = (float)pos.z + val; break;
        }
        vl[e] = p;
        nl[e] = nrm[a] + val * (nrm[bc] - nrm[a]);
        cl[e] = mc_color(c[a], c[bc], val);
      }
      // MarchingCube (MeshScene.cu:249-285)
      const int ntri = c_mc.nverts[ci] / 3;
      const uint32_t base = atomicAdd(count, (uint32_t)ntri);
      for (int j = 0; j < ntri; ++j) {
        const uint32_t tid = base + j;
        if (tid >= max_tri) return;
        for (int q = 0; q < 3; ++q) {
          const int e = c_mc.tri[ci][3 * j + q];
          const f3 v = vl[e] * vs;
          const f3 nn = nl[e];
          const float len = sqrtf(dot(nn, nn));
          vert[3 * (size_t)tid + q] = make_float3(v.x, v.y, v.z);
          norm[3 * (size_t)tid + q] = make_float3(nn.x / len, nn.y / len, nn.z / len);
          col[3 * (size_t)tid + q] = cl[e];
        }
      }
    }
  }
}

}  // namespace

void launch_mesh(const DevMap &m, float3 *vert, float3 *norm, uchar3 *col, uint32_t max_tri, uint32_t *count,
                 cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
  k_mesh<<<sms * 16, kMeshThreads, 0, s>>>(m, vert, norm, col, max_tri, count);
  note_launch();
}

}  // namespace sf
