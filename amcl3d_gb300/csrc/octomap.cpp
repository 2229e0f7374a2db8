// Octomap map files without the octomap library: openOcTree + computePointCloud
// (PointCloudTools.cpp:26-82) and Grid3d::open (Grid3d.cpp:25-78) behind the C ABI.
//
// octomap is a third-party dependency whose source is not in the reference tree.
// This reader follows its published file formats:
//  * header: first line "# Octomap OcTree binary file" (.bt) or "# Octomap OcTree
//    file" (.ot); then whitespace-separated tokens: '#' starts a comment line,
//    "id <type>", "size <nodes>", "res <metres>", unknown keywords skip their line,
//    "data" ends the header (the rest of its line is skipped).  id "1" is the old
//    name of "OcTree"; the id must be "OcTree" and res > 0.
//  * .bt body: per inner node two bytes (children 0-3, then 4-7), two bits per child
//    i at bit positions 2i and 2i+1: (1,0) free leaf, (0,1) occupied leaf, (1,1)
//    inner node whose own bytes follow depth first in child order, (0,0) none.  The
//    node count must equal the header's size.
//  * .ot body: per node a float32 log-odds value and a byte whose bit i marks child
//    i, then the children depth first; a node without children is a leaf, occupied
//    when its log-odds is >= 0 (occupancy probability 0.5).
//  * geometry: 16 levels below a root whose key is 32768 per axis; the child i of a
//    node at depth d - 1 has key parent + off on the axes whose bit of i is set and
//    parent - off - (off == 0) on the others, off = 32768 >> d.  A leaf centre is
//    (key - 32768 + 0.5) * res at depth 16, else
//    (floor((key - 32768) / 2^(16-d)) + 0.5) * res * 2^(16-d).  Leaves are visited
//    depth first in child order.
//  * computePointCloud keeps the (float) centres of the occupied leaves; the metric
//    bounds span every leaf, free ones included: min of centre - size/2, max of
//    (centre - size/2) + size.
// A truncated body is an error here (the octomap stream reader stops silently).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/amcl3d_gpu.h"

namespace amcl
{
int fail(int status, const std::string& msg);
}

namespace
{
constexpr int TREE_DEPTH = 16;
constexpr int32_t ROOT_KEY = 32768;

struct OctreeScan
{
  double res = 0.0;
  uint64_t nodes = 0;
  double mn[3], mx[3];
  std::vector<float> occ;  // x, y, z, 1 per occupied leaf
  std::string err;
};

double key_to_coord(int32_t key, int depth, double res)
{
  if (depth == 0)
    return 0.0;
  if (depth == TREE_DEPTH)
    return (static_cast<double>(key - ROOT_KEY) + 0.5) * res;
  const double span = static_cast<double>(1 << (TREE_DEPTH - depth));
  return (std::floor((static_cast<double>(key) - static_cast<double>(ROOT_KEY)) / span) + 0.5) * (res * span);
}

void child_key(const int32_t parent[3], int i, int depth, int32_t out[3])
{
  const int32_t off = ROOT_KEY >> depth;
  for (int a = 0; a < 3; ++a)
    out[a] = ((i >> a) & 1) ? parent[a] + off : parent[a] - off - (off ? 0 : 1);
}

void add_leaf(OctreeScan& T, const int32_t key[3], int depth, bool occupied)
{
  double c[3];
  const double size = T.res * static_cast<double>(1 << (TREE_DEPTH - depth));
  const double half = size / 2.0;
  for (int a = 0; a < 3; ++a)
  {
    c[a] = key_to_coord(key[a], depth, T.res);
    const double lo = c[a] - half;
    if (lo < T.mn[a])
      T.mn[a] = lo;
    const double hi = lo + size;
    if (hi > T.mx[a])
      T.mx[a] = hi;
  }
  if (occupied)
  {
    T.occ.push_back(static_cast<float>(c[0]));
    T.occ.push_back(static_cast<float>(c[1]));
    T.occ.push_back(static_cast<float>(c[2]));
    T.occ.push_back(1.0f);
  }
}

struct Cursor
{
  const unsigned char* p;
  const unsigned char* end;
};

bool read_bt_node(Cursor& c, OctreeScan& T, const int32_t key[3], int depth)
{
  if (depth >= TREE_DEPTH)
  {
    T.err = "inner node below the last tree level";
    return false;
  }
  if (c.end - c.p < 2)
  {
    T.err = "truncated tree";
    return false;
  }
  const unsigned char bytes[2] = { c.p[0], c.p[1] };
  c.p += 2;
  for (int i = 0; i < 8; ++i)
  {
    const unsigned b = bytes[i >> 2], j = static_cast<unsigned>(i & 3);
    const int lo = (b >> (2 * j)) & 1, hi = (b >> (2 * j + 1)) & 1;
    if (!lo && !hi)
      continue;
    T.nodes += 1;
    int32_t ck[3];
    child_key(key, i, depth + 1, ck);
    if (lo && !hi)
      add_leaf(T, ck, depth + 1, false);
    else if (!lo && hi)
      add_leaf(T, ck, depth + 1, true);
    else if (!read_bt_node(c, T, ck, depth + 1))
      return false;
  }
  return true;
}

// Returns false on error; *leaf_value receives the log-odds of a leaf, NAN for an inner node.
bool read_ot_node(Cursor& c, OctreeScan& T, const int32_t key[3], int depth, float* leaf_value)
{
  if (c.end - c.p < 5)
  {
    T.err = "truncated tree";
    return false;
  }
  float v;
  std::memcpy(&v, c.p, 4);
  const unsigned children = c.p[4];
  c.p += 5;
  if (!children)
  {
    *leaf_value = v;
    return true;
  }
  *leaf_value = std::numeric_limits<float>::quiet_NaN();
  if (depth >= TREE_DEPTH)
  {
    T.err = "inner node below the last tree level";
    return false;
  }
  for (int i = 0; i < 8; ++i)
  {
    if (!((children >> i) & 1))
      continue;
    T.nodes += 1;
    int32_t ck[3];
    child_key(key, i, depth + 1, ck);
    float cv;
    if (!read_ot_node(c, T, ck, depth + 1, &cv))
      return false;
    if (!std::isnan(cv))
      add_leaf(T, ck, depth + 1, cv >= 0.0f);
  }
  return true;
}

bool ends_with(const std::string& s, const char* ext)
{
  const size_t n = std::strlen(ext);
  return s.size() >= n && s.compare(s.size() - n, n, ext) == 0;
}

// The header's tokens; returns the offset of the body or 0 on error.
size_t parse_header(const std::vector<unsigned char>& b, const char* first, std::string& id, uint64_t& size,
                    double& res, std::string& err)
{
  size_t pos = 0;
  while (pos < b.size() && b[pos] != '\n')
    ++pos;
  if (pos >= b.size() || std::string(b.begin(), b.begin() + static_cast<long>(pos)).rfind(first, 0) != 0)
  {
    err = std::string("first line does not start with \"") + first + "\"";
    return 0;
  }
  ++pos;
  auto space = [](unsigned char ch) { return ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r' || ch == '\v' || ch == '\f'; };
  auto token = [&](size_t& p) {
    while (p < b.size() && space(b[p]))
      ++p;
    const size_t q0 = p;
    while (p < b.size() && !space(b[p]))
      ++p;
    return std::string(b.begin() + static_cast<long>(q0), b.begin() + static_cast<long>(p));
  };
  auto skip_line = [&](size_t& p) {
    while (p < b.size() && b[p] != '\n')
      ++p;
    if (p < b.size())
      ++p;
  };
  id.clear();
  size = 0;
  res = 0.0;
  while (true)
  {
    const std::string t = token(pos);
    if (t.empty())
    {
      err = "header without a data line";
      return 0;
    }
    if (t == "data")
    {
      skip_line(pos);
      break;
    }
    if (t[0] == '#')
      skip_line(pos);
    else if (t == "id")
      id = token(pos);
    else if (t == "res")
      res = std::strtod(token(pos).c_str(), nullptr);
    else if (t == "size")
      size = std::strtoull(token(pos).c_str(), nullptr, 10);
    else
      skip_line(pos);
  }
  if (id == "1")
    id = "OcTree";
  if (id.empty() || !(res > 0.0))
  {
    err = "header without an id or with res <= 0";
    return 0;
  }
  return pos;
}

// openOcTree + computePointCloud.  Returns AMCL_OK, AMCL_EIO (missing / unreadable
// file) or AMCL_EINVAL (not an OcTree, malformed, empty) with T.err set.
int scan_octree(const std::string& path, OctreeScan& T)
{
  const bool bt = ends_with(path, ".bt"), ot = ends_with(path, ".ot");
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f)
  {
    T.err = "Cannot find file " + path;
    return AMCL_EIO;
  }
  if (path.size() < 3)
  {
    std::fclose(f);
    T.err = "map path shorter than its extension";
    return AMCL_EINVAL;
  }
  std::vector<unsigned char> b;
  unsigned char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0)
    b.insert(b.end(), buf, buf + got);
  std::fclose(f);
  if (!bt && !ot)
  {
    T.err = "OcTree cannot be created from file " + path;
    return AMCL_EINVAL;
  }
  std::string id;
  uint64_t size = 0;
  const size_t body = parse_header(b, bt ? "# Octomap OcTree binary file" : "# Octomap OcTree file", id, size,
                                   T.res, T.err);
  if (!body)
    return AMCL_EINVAL;
  if (id != "OcTree")
  {
    T.err = "tree type " + id + " is not an OcTree";
    return AMCL_EINVAL;
  }
  for (int a = 0; a < 3; ++a)
  {
    T.mn[a] = std::numeric_limits<double>::max();
    T.mx[a] = -std::numeric_limits<double>::max();
  }
  T.nodes = 0;
  if (size > 0)
  {
    Cursor c{ b.data() + body, b.data() + b.size() };
    const int32_t root[3] = { ROOT_KEY, ROOT_KEY, ROOT_KEY };
    T.nodes = 1;
    bool ok;
    if (bt)
      ok = read_bt_node(c, T, root, 0);
    else
    {
      float v;
      ok = read_ot_node(c, T, root, 0, &v);
      if (ok && !std::isnan(v))
        add_leaf(T, root, 0, v >= 0.0f);
    }
    if (!ok)
      return AMCL_EINVAL;
  }
  if (bt && T.nodes != size)
  {
    T.err = "tree size mismatch: " + std::to_string(T.nodes) + " nodes read, " + std::to_string(size) + " declared";
    return AMCL_EINVAL;
  }
  if (T.nodes <= 1)
  {
    T.err = "OcTree is empty";
    return AMCL_EINVAL;
  }
  return AMCL_OK;
}
}  // namespace

extern "C" int amcl_octomap_read(const char* path, float* xyz4, uint64_t cap, uint64_t* n_points, double min[3],
                                 double max[3], double* resolution, uint64_t* tree_nodes)
{
  if (!path || !n_points || (cap && !xyz4))
    return amcl::fail(AMCL_EINVAL, "amcl_octomap_read: bad arguments");
  OctreeScan T;
  const int rc = scan_octree(path, T);
  if (rc)
    return amcl::fail(rc, "amcl_octomap_read: " + T.err);
  const uint64_t n = T.occ.size() / 4;
  *n_points = n;
  if (min && max)
    for (int a = 0; a < 3; ++a)
    {
      min[a] = T.mn[a];
      max[a] = T.mx[a];
    }
  if (resolution)
    *resolution = T.res;
  if (tree_nodes)
    *tree_nodes = T.nodes;
  if (xyz4)
  {
    if (n > cap)
      return amcl::fail(AMCL_ERANGE, "amcl_octomap_read: more occupied leaves than the output holds");
    std::memcpy(xyz4, T.occ.data(), n * 16);
  }
  return AMCL_OK;
}

extern "C" int amcl_grid_open(amcl_grid_t g, const char* map_path, double sensor_dev, uint64_t* n_points)
{
  if (!g || !map_path)
    return amcl::fail(AMCL_EINVAL, "amcl_grid_open: bad arguments");
  const std::string path(map_path);
  OctreeScan T;
  int rc = scan_octree(path, T);
  if (rc)
    return amcl::fail(rc, "amcl_grid_open: " + T.err);
  if (n_points)
    *n_points = T.occ.size() / 4;
  // The .grid cache beside the map (Grid3d.cpp:50-58): loaded when it matches.
  const std::string grid_path = path.substr(0, path.find(ends_with(path, ".bt") ? ".bt" : ".ot")) + ".grid";
  if (amcl_grid_load(g, grid_path.c_str(), T.mn, T.mx, T.res, sensor_dev) == AMCL_OK)
    return AMCL_OK;
  if ((rc = amcl_grid_build(g, T.occ.empty() ? nullptr : T.occ.data(), T.occ.size() / 4, 4, T.mn, T.mx, T.res,
                            sensor_dev)))
    return rc;
  amcl_grid_save(g, grid_path.c_str());  // Grid3d.cpp:77: a failed save is not an error
  return AMCL_OK;
}
