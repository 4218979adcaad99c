// Host driver for the reference's own device code compiled for the CPU by
// build_ref.py (test infrastructure only).  Calls the reference launchers
// (Tracking/Reduction.h, Mapping/RenderScene.h) on caller arrays, with a
// map laid out as Mapping::Create does (Mapping/Mapping.cc:11-51) and the
// DeviceMap view of Mapping::operator DeviceMap (Mapping.cc:363-377).
#include <cstring>
#include <vector>

#include "Constant.h"
#include "DeviceMap.h"
#include "Reduction.h"
#include "RenderScene.h"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

extern "C" void ref_unify_neighbor_impl(DeviceMap map, unsigned nvis);
extern "C" void ref_rgb_rows_impl(const unsigned char *, const unsigned char *, const float *, const float *,
                                  const short *, const short *, int, int, const float *, const float *,
                                  const float *, const float *, const float *, const float *, float, float,
                                  float, float, int *, float *, float *);
extern "C" void ref_icp_rows_impl(const float *, const float *, const float *, const float *, int, int,
                                  const float *, const float *, const float *, const float *,
                                  const float *, float, float, float, float, float *);

namespace {
Matrix3f m3(const float *R) {
  Matrix3f M;
  M.rowx = make_float3(R[0], R[1], R[2]);
  M.rowy = make_float3(R[3], R[4], R[5]);
  M.rowz = make_float3(R[6], R[7], R[8]);
  return M;
}
template <class T>
void up(DeviceArray2D<T> &a, const void *host, int cols, int rows) {
  a.create(cols, rows);
  a.upload(host, sizeof(T) * cols);
}
template <class T>
void down(const DeviceArray2D<T> &a, void *host) {
  a.download(host, sizeof(T) * a.cols);
}

struct RefMap {
  DeviceArray<int> heapCounter, hashCounter, heap, bucketMutex;
  DeviceArray<uint> noVisibleEntries, noRenderingBlocks;
  DeviceArray<Voxel> sdfBlock;
  DeviceArray<HashEntry> hashEntries, visibleEntries;
  DeviceArray2D<float> zRangeMin, zRangeMax;
  DeviceArray<RenderingBlock> renderingBlockList;
  uint noVisible = 0;

  RefMap() {
    heapCounter.create(1);
    hashCounter.create(1);
    noVisibleEntries.create(1);
    heap.create(DeviceMap::NumSdfBlocks);
    sdfBlock.create(DeviceMap::NumVoxels);
    bucketMutex.create(DeviceMap::NumBuckets);
    hashEntries.create(DeviceMap::NumEntries);
    visibleEntries.create(DeviceMap::NumEntries);
    zRangeMin.create(80, 60);
    zRangeMax.create(80, 60);
    noRenderingBlocks.create(1);
    renderingBlockList.create(DeviceMap::MaxRenderingBlocks);
    ResetMap(view());
  }
  DeviceMap view() const {
    DeviceMap map;
    map.heapMem = heap;
    map.heapCounter = heapCounter;
    map.noVisibleBlocks = noVisibleEntries;
    map.bucketMutex = bucketMutex;
    map.hashEntries = hashEntries;
    map.visibleEntries = visibleEntries;
    map.voxelBlocks = sdfBlock;
    map.entryPtr = hashCounter;
    return map;
  }
};
}  // namespace

extern "C" {

void ref_constants(double *out) {
  out[0] = DeviceMap::VoxelSize;
  out[1] = DeviceMap::TruncateDist;
  out[2] = DeviceMap::NumBuckets;
  out[3] = DeviceMap::NumExcess;
  out[4] = DeviceMap::NumSdfBlocks;
  out[5] = DeviceMap::DepthMin;
  out[6] = DeviceMap::DepthMax;
  out[7] = DeviceMap::stepScale;
}

void ref_filter_depth(const uint16_t *d, int cols, int rows, float scale, float cutoff, float *raw,
                      float *filt) {
  DeviceArray2D<unsigned short> dd;
  up(dd, d, cols, rows);
  DeviceArray2D<float> r(cols, rows), f(cols, rows);
  FilterDepth(dd, r, f, scale, cutoff);
  down(r, raw);
  down(f, filt);
}

void ref_pyrdown(const float *src, int sc, int sr, float *dst) {
  DeviceArray2D<float> s, o(sc / 2, sr / 2);
  up(s, src, sc, sr);
  PyrDownGauss(s, o);
  down(o, dst);
}

void ref_vmap(const float *depth, int cols, int rows, float fx, float fy, float cx, float cy,
              float cutoff, float *vmap) {
  DeviceArray2D<float> d;
  up(d, depth, cols, rows);
  DeviceArray2D<float4> v(cols, rows);
  ComputeVMap(d, v, fx, fy, cx, cy, cutoff);
  down(v, vmap);
}

void ref_nmap(const float *vmap, int cols, int rows, float *nmap) {
  DeviceArray2D<float4> v, n(cols, rows);
  up(v, vmap, cols, rows);
  ComputeNMap(v, n);
  down(n, nmap);
}

void ref_resize(const float *vsrc, const float *nsrc, int sc, int sr, float *vdst, float *ndst) {
  DeviceArray2D<float4> vs, ns, vd(sc / 2, sr / 2), nd(sc / 2, sr / 2);
  up(vs, vsrc, sc, sr);
  up(ns, nsrc, sc, sr);
  ResizeMap(vs, ns, vd, nd);
  down(vd, vdst);
  down(nd, ndst);
}

void ref_icp_rows(const float *vc, const float *vl, const float *nc, const float *nl, int cols, int rows,
                  const float *Rc, const float *tc, const float *Rl, const float *RlInv, const float *tl,
                  float fx, float fy, float cx, float cy, float *out29) {
  ref_icp_rows_impl(vc, vl, nc, nl, cols, rows, Rc, tc, Rl, RlInv, tl, fx, fy, cx, cy, out29);
}

// Frame::FillImages' intensity part (Core/Frame.cc:74-84): ImageToIntensity,
// PyrDownGauss(unsigned char), ComputeDerivativeImage.
void ref_intensity(const uint8_t *rgb, int cols, int rows, uint8_t *out) {
  DeviceArray2D<uchar3> c;
  up(c, rgb, cols, rows);
  DeviceArray2D<unsigned char> o(cols, rows);
  ImageToIntensity(c, o);
  down(o, out);
}

void ref_pyrdown_u8(const uint8_t *src, int sc, int sr, uint8_t *dst) {
  DeviceArray2D<unsigned char> s, o(sc / 2, sr / 2);
  up(s, src, sc, sr);
  PyrDownGauss(s, o);
  down(o, dst);
}

void ref_sobel(const uint8_t *img, int cols, int rows, int16_t *dx, int16_t *dy) {
  DeviceArray2D<unsigned char> i;
  up(i, img, cols, rows);
  DeviceArray2D<short> x(cols, rows), y(cols, rows);
  ComputeDerivativeImage(i, x, y);
  down(x, dx);
  down(y, dy);
}

void ref_rgb_rows(const uint8_t *inext, const uint8_t *ilast, const float *vn, const float *vl, const int16_t *dx,
                  const int16_t *dy, int cols, int rows, const float *Rc, const float *RcI, const float *Rl,
                  const float *RlI, const float *tc, const float *tl, float fx, float fy, float cx, float cy,
                  int *res2, float *sigma, float *out29) {
  ref_rgb_rows_impl(inext, ilast, vn, vl, dx, dy, cols, rows, Rc, RcI, Rl, RlI, tc, tl, fx, fy, cx, cy, res2,
                    sigma, out29);
}

void *ref_map_create() { return new RefMap(); }
void ref_map_destroy(void *m) { delete (RefMap *)m; }

// Mapping::FuseColor -> FuseMapColor (Mapping.cc:76-97): depth/max from
// DeviceMap, intrinsics of level 0.
unsigned ref_map_fuse(void *mp, const float *depth, const uint8_t *rgb, const float *nmap,
                      const uint8_t *mask, int num_detection, int cols, int rows, const float *R,
                      const float *Rinv, const float *t, float fx, float fy, float cx, float cy) {
  RefMap &m = *(RefMap *)mp;
  DeviceArray2D<float> d;
  DeviceArray2D<uchar3> c;
  DeviceArray2D<float4> n;
  DeviceArray2D<unsigned char> mk;
  up(d, depth, cols, rows);
  up(c, rgb, cols, rows);
  up(n, nmap, cols, rows);
  up(mk, mask, cols, rows);
  DeviceArray<int> labels(1);
  uint host = 0;
  FuseMapColor(d, c, n, mk, labels, num_detection, m.noVisibleEntries, m3(R), m3(Rinv),
               make_float3(t[0], t[1], t[2]), m.view(), fx, fy, cx, cy, DeviceMap::DepthMax,
               DeviceMap::DepthMin, &host);
  m.noVisible = host;
  return host;
}

unsigned ref_map_visibility(void *mp, const float *R, const float *Rinv, const float *t, int cols, int rows,
                            float fx, float fy, float cx, float cy) {
  RefMap &m = *(RefMap *)mp;
  uint host = 0;
  CheckBlockVisibility(m.view(), m.noVisibleEntries, m3(R), m3(Rinv), make_float3(t[0], t[1], t[2]), cols,
                       rows, fx, fy, cx, cy, DeviceMap::DepthMax, DeviceMap::DepthMin, &host);
  m.noVisible = host;
  return host;
}

void ref_map_semantics(void *mp, const float *depth, const uint8_t *rgb, const float *nmap, const uint8_t *mask,
                       int num_detection, int cols, int rows, const float *R, const float *Rinv, const float *t,
                       float fx, float fy, float cx, float cy) {
  RefMap &m = *(RefMap *)mp;
  DeviceArray2D<float> d;
  DeviceArray2D<uchar3> c;
  DeviceArray2D<float4> n;
  DeviceArray2D<unsigned char> mk;
  up(d, depth, cols, rows);
  up(c, rgb, cols, rows);
  up(n, nmap, cols, rows);
  up(mk, mask, cols, rows);
  DeviceArray<int> labels(1);
  AnalyzeMapSemantics(d, c, n, mk, labels, num_detection, m.noVisibleEntries, m3(R), m3(Rinv),
                      make_float3(t[0], t[1], t[2]), m.view(), fx, fy, cx, cy, DeviceMap::DepthMax,
                      DeviceMap::DepthMin);
}

// Mapping::RayTrace (Mapping.cc:142-161).  The rendering-block list starts
// as empty tiles so that fillBlocks' reads past the count (RenderScene.cu
// :173, :281) touch nothing.  zmin/zmax: 80 x 60 floats.
int ref_map_raytrace(void *mp, int cols, int rows, const float *R, const float *Rinv, const float *t, float fx,
                     float fy, float cx, float cy, float *zmin, float *zmax, unsigned *nblocks, float *vmap,
                     float *nmap) {
  RefMap &m = *(RefMap *)mp;
  RenderingBlock empty;
  empty.upperLeft = make_short2(32767, 32767);
  empty.lowerRight = make_short2(-1, -1);
  empty.zRange = make_float2(0, 0);
  std::vector<RenderingBlock> init(DeviceMap::MaxRenderingBlocks, empty);
  m.renderingBlockList.upload(init.data());
  DeviceArray2D<float4> v(cols, rows), n(cols, rows);
  v.upload(vmap, sizeof(float4) * cols);  // the frame's own maps when nothing renders
  n.upload(nmap, sizeof(float4) * cols);
  bool ok = CreateRenderingBlocks(m.visibleEntries, m.zRangeMin, m.zRangeMax, DeviceMap::DepthMax,
                                  DeviceMap::DepthMin, m.renderingBlockList, m.noRenderingBlocks, m3(Rinv),
                                  make_float3(t[0], t[1], t[2]), m.noVisible, fx, fy, cx, cy);
  uint nb = 0;
  m.noRenderingBlocks.download(&nb);
  *nblocks = nb;
  m.zRangeMin.download(zmin, sizeof(float) * 80);
  m.zRangeMax.download(zmax, sizeof(float) * 80);
  if (ok)
    Raycast(m.view(), v, n, m.zRangeMin, m.zRangeMax, m3(R), m3(Rinv), make_float3(t[0], t[1], t[2]),
            1.0 / fx, 1.0 / fy, cx, cy);
  down(v, vmap);
  down(n, nmap);
  return ok ? 1 : 0;
}

const void *ref_map_entries(void *mp) { return ((RefMap *)mp)->hashEntries.data; }
const void *ref_map_visible(void *mp) { return ((RefMap *)mp)->visibleEntries.data; }
const void *ref_map_voxels(void *mp) { return ((RefMap *)mp)->sdfBlock.data; }
// Mapping::CreateModel (Mapping.cc:183-192): MeshScene with the tables of
// Constant.h.  Returns the triangle count; vert / nrm float[9] and col
// uint8[9] per triangle (up to max_tri).
unsigned ref_map_mesh(void *mp, unsigned max_tri, float *vert, float *nrm, uint8_t *col) {
  RefMap &m = *(RefMap *)mp;
  DeviceArray<int> edge(256), verts(256);
  DeviceArray2D<int> tri(16, 256);
  edge.upload(edgeTableHost, 256);
  verts.upload(vertexTableHost, 256);
  tri.upload(triangleTableHost, 16 * sizeof(int));
  DeviceArray<float3> normal(DeviceMap::MaxVertices), vertex(DeviceMap::MaxVertices);
  DeviceArray<uchar3> color(DeviceMap::MaxVertices);
  DeviceArray<int3> blocks(DeviceMap::NumEntries);
  DeviceArray<uint> nblocks(1), ntri(1);
  uint n = MeshScene(nblocks, ntri, m.view(), edge, verts, tri, normal, vertex, color, blocks);
  if (n > max_tri) n = max_tri;
  vertex.download(vert, 3 * n);
  normal.download(nrm, 3 * n);
  color.download(col, 3 * n);
  return n;
}

// UnifyNeighborKernel over hash slots [0, nvis) with the (8, 8) block of
// AnalyzeMapSemantics (FuseMap.cu:1244-1246).
void ref_map_unify(void *mp, unsigned nvis) {
  RefMap &m = *(RefMap *)mp;
  ref_unify_neighbor_impl(m.view(), nvis);
}

void ref_map_counters(void *mp, int *out) {
  RefMap &m = *(RefMap *)mp;
  m.heapCounter.download(out + 0);
  m.hashCounter.download(out + 1);
  out[2] = (int)m.noVisible;
  int alloc = 0;
  const HashEntry *e = (const HashEntry *)m.hashEntries.data;
  for (uint i = 0; i < DeviceMap::NumEntries; ++i) alloc += e[i].ptr >= 0;
  out[3] = alloc;
}

}  // extern "C"
