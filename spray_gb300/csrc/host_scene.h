// Host-side scene description, `.spray` scene-file parser, PLY reader/writer
// and the wavelet isosurface generator used to build the benchmark scenes.
//
// The parser keeps SpRay's scene grammar (src/io/scene_loader.cc:42-358):
//   light point px py pz r g b | light diffuse r g b
//   domain / file <ply> / mtl diffuse|mirror|glass|transmission ... /
//   bound minx miny minz maxx maxy maxz / scale / rotate x|y|z deg /
//   translate / face N / vertex N / # comment
// The world AABB of a domain is its transform applied to the two object-space
// bound corners (scene_loader.cc:351-357), which is what SpRay's domain
// scheduler tests rays against.  PLY reading follows src/io/ply_loader.cc:179-324
// (ascii or binary little endian, float xyz, optional uchar rgb, face lists).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sg {

struct Mat4 {  // column-major, m[col][row] like the 4x4 transform in SpRay
  float m[4][4];
  static Mat4 identity();
  bool isIdentity() const;
};

Mat4 translate(const Mat4& m, float x, float y, float z);
Mat4 scale(const Mat4& m, float x, float y, float z);
Mat4 rotate(const Mat4& m, float radians, int axis);
void transformPoint(const Mat4& m, const float in[3], float out[3]);

enum BsdfType { BSDF_DIFFUSE = 0, BSDF_MIRROR = 1, BSDF_GLASS = 2, BSDF_TRANSMISSION = 3 };
enum LightType { LIGHT_POINT = 0, LIGHT_DIFFUSE = 1, LIGHT_QUAD = 2 };

struct Light {
  int type = LIGHT_POINT;
  float position[3] = {0, 0, 0};
  float radiance[3] = {0, 0, 0};
  float edge1[3] = {0, 0, 0};  // quad lights only (extension)
  float edge2[3] = {0, 0, 0};
};

struct Domain {
  int id = -1;
  std::string filename;
  int bsdf_type = BSDF_DIFFUSE;
  float bsdf_params[3] = {1, 1, 1};
  float object_bounds[6] = {0, 0, 0, 0, 0, 0};
  float world_bounds[6] = {0, 0, 0, 0, 0, 0};
  uint64_t num_vertices = 0;  // as declared by the scene file
  uint64_t num_faces = 0;
  Mat4 transform = Mat4::identity();
};

struct SceneDesc {
  std::vector<Domain> domains;
  std::vector<Light> lights;
};

// Mesh of one domain after loading (vertices in world space).
struct Mesh {
  std::vector<float> vertices;   // 3 * nv
  std::vector<uint32_t> faces;   // 3 * nf
  std::vector<uint32_t> colors;  // nv, packed 0x00RRGGBB
  bool has_color = false;
};

// Parse a .spray file; ply_path is prepended to each "file" entry when not
// empty.  Throws std::runtime_error with a message on malformed input.
SceneDesc loadSceneFile(const std::string& filename, const std::string& ply_path);

// Read a PLY file into mesh (object space).
void readPly(const std::string& filename, Mesh* mesh);

// Load a domain's PLY and apply its transform when it is not the identity
// (src/render/scene.inl:177-181, trimesh_buffer.cc:141-157).
void loadDomainMesh(const Domain& d, Mesh* mesh);

// Write a binary little endian PLY with float xyz, uchar rgb and
// "list uchar int vertex_indices" faces.
void writePly(const std::string& filename, const float* v, uint64_t nv,
              const uint32_t* colors, const uint32_t* f, uint64_t nf);

// Wavelet field f = 255*exp(-(x^2+y^2+z^2)/(2*0.5^2)) + 10*sin(60x+p0)
//                 + 18*sin(30y+p1) + 5*cos(40z+p2) on [-1,1]^3.
struct WaveletSpec {
  int samples = 64;        // grid points per axis
  double iso = 157.0;
  double phase[3] = {0, 0, 0};
};

// Marching-cubes isosurface of the wavelet field.  Cells are polygonised
// without a case table: every cube face contributes oriented segments between
// its sign-changing edges (ambiguous faces decided by the mean of the face's
// corners), the segments are linked into loops and each loop is fanned into
// triangles.  Vertices are shared between neighbouring cells.
void generateWavelet(const WaveletSpec& spec, std::vector<float>* vertices,
                     std::vector<uint32_t>* faces);

}  // namespace sg
