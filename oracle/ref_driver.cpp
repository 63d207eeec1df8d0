/*
 * extern "C" driver around the reference kvs::MarchingCubes, linked with the
 * reference's own sources by oracle/Makefile.ref into oracle/_ref/.
 *
 * Test infrastructure only.  It builds a kvs::StructuredVolumeObject from a
 * raw buffer, runs the reference mapper through its public constructor
 * (Source/Core/Visualization/Mapper/MarchingCubes.cpp:25-37), and copies the
 * resulting kvs::PolygonObject arrays out so Python (ctypes) can compare them
 * with the C restatement and write golden fixtures.
 */
#include <kvs/StructuredVolumeObject>
#include <kvs/UnstructuredVolumeObject>
#include <kvs/MarchingTetrahedra>
#include <kvs/MarchingHexahedra>
#include <kvs/MarchingPyramid>
#include <kvs/MarchingPrism>
#include <kvs/PolygonObject>
#include <kvs/MarchingCubes>
#include <kvs/Isosurface>
#include <kvs/PolygonExporter>
#include <kvs/Stl>
#include <kvs/KVSMLPolygonObject>
#include <kvs/Ply>
#include <kvs/AVSField>
#include <kvs/SlicePlane>
#include <kvs/TransferFunction>
#include <kvs/HydrogenVolumeData>
#include <kvs/ValueArray>
#include <kvs/AnyValueArray>
#include <chrono>
#include <cstdlib>
#include <cstring>

extern "C" {

struct kvsref_result
{
    int success;
    unsigned long long ncoords;      // number of floats in coords
    unsigned long long nnormals;     // number of floats in normals
    unsigned long long nconnections; // number of uint32 in connections
    unsigned long long ncolors;      // number of bytes in colors
    unsigned long long nopacities;   // number of bytes in opacities
    float* coords;
    float* normals;
    unsigned int* connections;
    unsigned char* colors;
    unsigned char* opacities;
    int polygon_type;
    int normal_type;
    int color_type;
    int vol_has_minmax;
    double vol_min;
    double vol_max;
    float min_obj[3], max_obj[3], min_ext[3], max_ext[3];
    double seconds;
};

} // extern "C"

namespace
{

template <typename T>
kvs::AnyValueArray MakeValues( const void* p, size_t n )
{
    return kvs::AnyValueArray( kvs::ValueArray<T>( static_cast<const T*>( p ), n ) );
}

// dtype codes follow the order of the reference's type switch
// (MarchingCubes.cpp:115-124): i8 i16 i32 i64 u8 u16 u32 u64 f32 f64.
kvs::AnyValueArray Values( int dtype, const void* p, size_t n )
{
    switch ( dtype )
    {
    case 0: return MakeValues<kvs::Int8>( p, n );
    case 1: return MakeValues<kvs::Int16>( p, n );
    case 2: return MakeValues<kvs::Int32>( p, n );
    case 3: return MakeValues<kvs::Int64>( p, n );
    case 4: return MakeValues<kvs::UInt8>( p, n );
    case 5: return MakeValues<kvs::UInt16>( p, n );
    case 6: return MakeValues<kvs::UInt32>( p, n );
    case 7: return MakeValues<kvs::UInt64>( p, n );
    case 8: return MakeValues<kvs::Real32>( p, n );
    case 9: return MakeValues<kvs::Real64>( p, n );
    default: return kvs::AnyValueArray();
    }
}

template <typename T>
T* CopyOut( const kvs::ValueArray<T>& a, unsigned long long* n )
{
    *n = a.size();
    if ( a.size() == 0 ) return nullptr;
    T* p = static_cast<T*>( std::malloc( a.size() * sizeof( T ) ) );
    std::memcpy( p, a.data(), a.size() * sizeof( T ) );
    return p;
}

void Copy3( float* dst, const kvs::Vec3& v ) { dst[0] = v.x(); dst[1] = v.y(); dst[2] = v.z(); }

// The arrays, types and bounding box of a mapper's PolygonObject, and the
// volume's min/max cache afterwards.
void Fill( const kvs::MapperBase* mapper, const kvs::PolygonObject* p, const kvs::VolumeObjectBase* vol,
           kvsref_result* out )
{
    out->success = mapper->isSuccess() ? 1 : 0;
    out->coords = CopyOut( p->coords(), &out->ncoords );
    out->normals = CopyOut( p->normals(), &out->nnormals );
    out->connections = CopyOut( p->connections(), &out->nconnections );
    out->colors = CopyOut( p->colors(), &out->ncolors );
    out->opacities = CopyOut( p->opacities(), &out->nopacities );
    out->polygon_type = int( p->polygonType() );
    out->normal_type = int( p->normalType() );
    out->color_type = int( p->colorType() );
    out->vol_has_minmax = vol->hasMinMaxValues() ? 1 : 0;
    out->vol_min = vol->minValue();
    out->vol_max = vol->maxValue();
    Copy3( out->min_obj, p->minObjectCoord() );
    Copy3( out->max_obj, p->maxObjectCoord() );
    Copy3( out->min_ext, p->minExternalCoord() );
    Copy3( out->max_ext, p->maxExternalCoord() );
}

} // namespace

extern "C" {

/*
 * grid_type: 0 uniform, 1 rectilinear (rect_coords = nx+ny+nz floats).
 * has_obj_coords: preset the volume's min/max object coords.
 * has_minmax: preset the volume's min/max values (skips the reference scan).
 * tf_has_range: give the transfer function a range before the call.
 * repeat: run the constructor this many times on fresh volume objects and
 *         report the fastest (for the CPU baseline); outputs are the last run's.
 */
int kvsref_marching_cubes(
    int dtype, const void* values, unsigned nx, unsigned ny, unsigned nz,
    double isolevel, int normal_type, int duplication,
    int has_minmax, double vmin, double vmax,
    int grid_type, const float* rect_coords,
    int has_obj_coords, const float* min_obj, const float* max_obj,
    int tf_resolution, int tf_has_range, float tf_min, float tf_max,
    int repeat, kvsref_result* out )
{
    std::memset( out, 0, sizeof( *out ) );
    const size_t n = size_t( nx ) * ny * nz;
    kvs::AnyValueArray vals = Values( dtype, values, n );
    if ( vals.size() != n ) return -1;

    kvs::TransferFunction tfunc( tf_resolution > 0 ? tf_resolution : 256 );
    if ( tf_has_range ) tfunc.setRange( tf_min, tf_max );

    const auto ntype = normal_type == 0 ? kvs::PolygonObject::PolygonNormal : kvs::PolygonObject::VertexNormal;
    if ( repeat < 1 ) repeat = 1;
    double best = 1e300;
    kvs::MarchingCubes* mc = nullptr;
    kvs::StructuredVolumeObject* vol = nullptr;
    for ( int r = 0; r < repeat; ++r )
    {
        delete mc; mc = nullptr;
        delete vol;
        vol = new kvs::StructuredVolumeObject();
        vol->setVeclen( 1 );
        vol->setResolution( kvs::Vec3ui( nx, ny, nz ) );
        vol->setValues( vals );
        if ( grid_type == 1 )
        {
            vol->setGridTypeToRectilinear();
            vol->setCoords( kvs::ValueArray<kvs::Real32>( rect_coords, size_t( nx ) + ny + nz ) );
        }
        else
        {
            vol->setGridTypeToUniform();
        }
        if ( has_obj_coords )
        {
            vol->setMinMaxObjectCoords( kvs::Vec3( min_obj[0], min_obj[1], min_obj[2] ),
                                        kvs::Vec3( max_obj[0], max_obj[1], max_obj[2] ) );
        }
        if ( has_minmax ) vol->setMinMaxValues( vmin, vmax );

        const auto t0 = std::chrono::steady_clock::now();
        mc = new kvs::MarchingCubes( vol, isolevel, ntype, duplication != 0, tfunc );
        const auto t1 = std::chrono::steady_clock::now();
        const double s = std::chrono::duration<double>( t1 - t0 ).count();
        if ( s < best ) best = s;
    }

    Fill( mc, mc, vol, out );
    out->seconds = best;
    delete mc;
    delete vol;
    return 0;
}

/*
 * The reference kvs::SlicePlane (Source/Core/Visualization/Mapper/SlicePlane.cpp)
 * on a uniform structured volume: form 0 SlicePlane( volume, coefficients, tf ),
 * form 1 SlicePlane( volume, point, normal, tf ) (plane[0..2] point,
 * plane[3..5] normal); has_obj_coords presets the volume's min/max object
 * coords.
 */
int kvsref_slice_plane(
    int form, int dtype, const void* values, unsigned nx, unsigned ny, unsigned nz, const float* plane,
    int has_minmax, double vmin, double vmax, int tf_resolution, int tf_has_range, float tf_min, float tf_max,
    int has_obj_coords, const float* min_obj, const float* max_obj, kvsref_result* out )
{
    std::memset( out, 0, sizeof( *out ) );
    const size_t n = size_t( nx ) * ny * nz;
    kvs::AnyValueArray vals = Values( dtype, values, n );
    if ( vals.size() != n ) return -1;
    kvs::TransferFunction tfunc( tf_resolution > 0 ? tf_resolution : 256 );
    if ( tf_has_range ) tfunc.setRange( tf_min, tf_max );
    auto* vol = new kvs::StructuredVolumeObject();
    vol->setVeclen( 1 );
    vol->setResolution( kvs::Vec3ui( nx, ny, nz ) );
    vol->setValues( vals );
    vol->setGridTypeToUniform();
    if ( has_minmax ) vol->setMinMaxValues( vmin, vmax );
    if ( has_obj_coords )
    {
        vol->setMinMaxObjectCoords( kvs::Vec3( min_obj[0], min_obj[1], min_obj[2] ),
                                    kvs::Vec3( max_obj[0], max_obj[1], max_obj[2] ) );
    }
    kvs::SlicePlane* s = nullptr;
    if ( form == 0 ) s = new kvs::SlicePlane( vol, kvs::Vec4( plane[0], plane[1], plane[2], plane[3] ), tfunc );
    else s = new kvs::SlicePlane( vol, kvs::Vec3( plane[0], plane[1], plane[2] ),
                                  kvs::Vec3( plane[3], plane[4], plane[5] ), tfunc );
    Fill( s, s, vol, out );
    delete s;
    delete vol;
    return 0;
}

/* kvs::SlicePlane on an UnstructuredVolumeObject (cell_type as in
 * kvsref_marching_cells); form 0: plane = a, b, c, d; form 1: plane = point,
 * normal. */
int kvsref_slice_cells(
    int form, int cell_type, int dtype, const void* values, unsigned long long nnodes, const float* coords,
    const unsigned int* connections, unsigned long long ncells, const float* plane, int has_minmax, double vmin,
    double vmax, int tf_resolution, int tf_has_range, float tf_min, float tf_max, kvsref_result* out )
{
    std::memset( out, 0, sizeof( *out ) );
    static const kvs::UnstructuredVolumeObject::CellType types[4] = {
        kvs::UnstructuredVolumeObject::Tetrahedra, kvs::UnstructuredVolumeObject::Hexahedra,
        kvs::UnstructuredVolumeObject::Pyramid, kvs::UnstructuredVolumeObject::Prism };
    static const size_t npc[4] = { 4, 8, 5, 6 };
    if ( cell_type < 0 || cell_type > 3 ) return -1;
    kvs::AnyValueArray vals = Values( dtype, values, nnodes );
    if ( vals.size() != nnodes ) return -1;
    kvs::TransferFunction tfunc( tf_resolution > 0 ? tf_resolution : 256 );
    if ( tf_has_range ) tfunc.setRange( tf_min, tf_max );
    auto* vol = new kvs::UnstructuredVolumeObject();
    vol->setCellType( types[cell_type] );
    vol->setVeclen( 1 );
    vol->setNumberOfNodes( nnodes );
    vol->setNumberOfCells( ncells );
    vol->setCoords( kvs::ValueArray<kvs::Real32>( coords, 3 * nnodes ) );
    vol->setConnections( kvs::ValueArray<kvs::UInt32>( connections, npc[cell_type] * ncells ) );
    vol->setValues( vals );
    if ( has_minmax ) vol->setMinMaxValues( vmin, vmax );
    kvs::SlicePlane* s = nullptr;
    if ( form == 0 ) s = new kvs::SlicePlane( vol, kvs::Vec4( plane[0], plane[1], plane[2], plane[3] ), tfunc );
    else s = new kvs::SlicePlane( vol, kvs::Vec3( plane[0], plane[1], plane[2] ),
                                  kvs::Vec3( plane[3], plane[4], plane[5] ), tfunc );
    Fill( s, s, vol, out );
    delete s;
    delete vol;
    return 0;
}

/*
 * KVSML structured volumes through the reference's own reader and writer
 * (StructuredVolumeObject::read / write, StructuredVolumeObject.cpp:171-270,
 * KVSMLStructuredVolumeObject).  write: writing type from (ascii, external).
 */
int kvsref_write_kvsml( int dtype, const void* values, unsigned nx, unsigned ny, unsigned nz, const char* path,
                        int ascii, int external, int has_minmax, double vmin, double vmax,
                        int has_obj, const float* min_obj, const float* max_obj )
{
    const size_t n = size_t( nx ) * ny * nz;
    kvs::StructuredVolumeObject vol;
    vol.setVeclen( 1 );
    vol.setResolution( kvs::Vec3ui( nx, ny, nz ) );
    vol.setValues( Values( dtype, values, n ) );
    vol.setGridTypeToUniform();
    if ( has_obj )
    {
        vol.setMinMaxObjectCoords( kvs::Vec3( min_obj[0], min_obj[1], min_obj[2] ),
                                   kvs::Vec3( max_obj[0], max_obj[1], max_obj[2] ) );
        vol.setMinMaxExternalCoords( kvs::Vec3( min_obj[0], min_obj[1], min_obj[2] ),
                                     kvs::Vec3( max_obj[0], max_obj[1], max_obj[2] ) );
    }
    else
    {
        vol.updateMinMaxCoords();
    }
    if ( has_minmax ) vol.setMinMaxValues( vmin, vmax );
    else vol.updateMinMaxValues();
    return vol.write( path, ascii != 0, external != 0 ) ? 0 : -1;
}

struct kvsref_volume
{
    int success;
    int dtype;               // -1: a type outside the ten of the mapper's switch
    unsigned nx, ny, nz;
    unsigned veclen;
    int grid_type;
    double vmin, vmax;
    float min_obj[3], max_obj[3], min_ext[3], max_ext[3];
    unsigned long long nbytes;
    unsigned char* values;   // malloc'ed copy, nbytes
};

int kvsref_read_kvsml( const char* path, kvsref_volume* out )
{
    std::memset( out, 0, sizeof( *out ) );
    kvs::StructuredVolumeObject vol;
    if ( !vol.read( path ) ) return -1;
    out->success = 1;
    const auto t = vol.values().typeID();
    static const kvs::Type::TypeID order[10] = {
        kvs::Type::TypeInt8, kvs::Type::TypeInt16, kvs::Type::TypeInt32, kvs::Type::TypeInt64,
        kvs::Type::TypeUInt8, kvs::Type::TypeUInt16, kvs::Type::TypeUInt32, kvs::Type::TypeUInt64,
        kvs::Type::TypeReal32, kvs::Type::TypeReal64 };
    out->dtype = -1;
    for ( int i = 0; i < 10; ++i ) if ( order[i] == t ) out->dtype = i;
    out->nx = vol.resolution().x(); out->ny = vol.resolution().y(); out->nz = vol.resolution().z();
    out->veclen = vol.veclen();
    out->grid_type = int( vol.gridType() );
    out->vmin = vol.minValue();
    out->vmax = vol.maxValue();
    Copy3( out->min_obj, vol.minObjectCoord() );
    Copy3( out->max_obj, vol.maxObjectCoord() );
    Copy3( out->min_ext, vol.minExternalCoord() );
    Copy3( out->max_ext, vol.maxExternalCoord() );
    out->nbytes = vol.values().byteSize();
    out->values = static_cast<unsigned char*>( std::malloc( out->nbytes ? out->nbytes : 1 ) );
    std::memcpy( out->values, vol.values().data(), out->nbytes );
    return 0;
}

void kvsref_free_volume( kvsref_volume* v ) { std::free( v->values ); std::memset( v, 0, sizeof( *v ) ); }

/*
 * An AVS field file read by kvs::AVSField (FileFormat/AVSField/AVSField.cpp)
 * and turned into a volume the way StructuredVolumeImporter::import(const
 * AVSField*) does (Visualization/Importer/StructuredVolumeImporter.cpp:155-189;
 * restated here because the importer's other formats pull in DICOM and more):
 * uniform fields only, object coords [0, dim - 1], external coords min_ext /
 * max_ext or the object coords, min/max by updateMinMaxValues.
 */
int kvsref_read_avs( const char* path, kvsref_volume* out )
{
    std::memset( out, 0, sizeof( *out ) );
    kvs::AVSField field( path );
    if ( field.isFailure() ) return -1;
    if ( field.fieldType() != kvs::AVSField::Uniform ) return -2;
    kvs::StructuredVolumeObject vol;
    const kvs::Vec3 min_obj( 0.0f, 0.0f, 0.0f );
    const kvs::Vec3 max_obj( float( field.dim().x() ) - 1.0f, float( field.dim().y() ) - 1.0f,
                             float( field.dim().z() ) - 1.0f );
    vol.setMinMaxObjectCoords( min_obj, max_obj );
    if ( field.hasMinMaxExt() ) vol.setMinMaxExternalCoords( field.minExt(), field.maxExt() );
    else vol.setMinMaxExternalCoords( min_obj, max_obj );
    vol.setGridType( kvs::StructuredVolumeObject::Uniform );
    vol.setVeclen( field.veclen() );
    vol.setResolution( field.dim() );
    vol.setValues( field.values() );
    vol.updateMinMaxValues();
    out->success = 1;
    const auto t = vol.values().typeID();
    static const kvs::Type::TypeID order[10] = {
        kvs::Type::TypeInt8, kvs::Type::TypeInt16, kvs::Type::TypeInt32, kvs::Type::TypeInt64,
        kvs::Type::TypeUInt8, kvs::Type::TypeUInt16, kvs::Type::TypeUInt32, kvs::Type::TypeUInt64,
        kvs::Type::TypeReal32, kvs::Type::TypeReal64 };
    out->dtype = -1;
    for ( int i = 0; i < 10; ++i ) if ( order[i] == t ) out->dtype = i;
    out->nx = vol.resolution().x(); out->ny = vol.resolution().y(); out->nz = vol.resolution().z();
    out->veclen = vol.veclen();
    out->grid_type = int( vol.gridType() );
    out->vmin = vol.minValue();
    out->vmax = vol.maxValue();
    Copy3( out->min_obj, vol.minObjectCoord() );
    Copy3( out->max_obj, vol.maxObjectCoord() );
    Copy3( out->min_ext, vol.minExternalCoord() );
    Copy3( out->max_ext, vol.maxExternalCoord() );
    out->nbytes = vol.values().byteSize();
    out->values = static_cast<unsigned char*>( std::malloc( out->nbytes ? out->nbytes : 1 ) );
    std::memcpy( out->values, vol.values().data(), out->nbytes );
    return 0;
}

/*
 * kvs::MarchingCubes on a uniform volume, then the reference's binary STL export
 * of the result: PolygonExporter<kvs::Stl>::exec (PolygonExporter.cpp:78-176)
 * and Stl::write with the Binary file type (Stl.cpp:170-199, 490-540).
 * Returns 0 when the file was written.
 */
int kvsref_marching_cubes_stl(
    int dtype, const void* values, unsigned nx, unsigned ny, unsigned nz,
    double isolevel, int normal_type, int duplication, const char* path )
{
    const size_t n = size_t( nx ) * ny * nz;
    kvs::AnyValueArray vals = Values( dtype, values, n );
    if ( vals.size() != n ) return -1;
    kvs::TransferFunction tfunc( 256 );
    const auto ntype = normal_type == 0 ? kvs::PolygonObject::PolygonNormal : kvs::PolygonObject::VertexNormal;
    auto* vol = new kvs::StructuredVolumeObject();
    vol->setVeclen( 1 );
    vol->setResolution( kvs::Vec3ui( nx, ny, nz ) );
    vol->setValues( vals );
    vol->setGridTypeToUniform();
    auto* mc = new kvs::MarchingCubes( vol, isolevel, ntype, duplication != 0, tfunc );
    kvs::PolygonExporter<kvs::Stl> exporter( mc );   // the exporter's one constructor runs exec
    int rc = -2;
    if ( exporter.kvs::ExporterBase::isSuccess() )
    {
        exporter.setFileType( kvs::Stl::Binary );
        rc = exporter.write( path ) ? 0 : -3;
    }
    delete mc;
    delete vol;
    return rc;
}

/*
 * kvs::MarchingCubes on a uniform volume with the default TransferFunction(256),
 * then one of the reference's polygon writers on the result:
 *   format 0: PolygonExporter<kvs::Stl> + Stl::write, Binary (Stl.cpp:490-540)
 *   format 1: PolygonExporter<kvs::Stl> + Stl::write, Ascii, the Stl default
 *             (Stl.cpp:86, 447-480)
 *   format 2/3/4: PolygonExporter<kvs::KVSMLPolygonObject> (PolygonExporter.cpp:22-68)
 *             + KVSMLPolygonObject::write (KVSMLPolygonObject.cpp:349-492) with
 *             the Ascii / ExternalAscii / ExternalBinary writing data type
 * Returns 0 when the file (and its external data files) were written.
 */
int kvsref_marching_cubes_export(
    int dtype, const void* values, unsigned nx, unsigned ny, unsigned nz,
    double isolevel, int normal_type, int duplication, int format, const char* path )
{
    const size_t n = size_t( nx ) * ny * nz;
    kvs::AnyValueArray vals = Values( dtype, values, n );
    if ( vals.size() != n ) return -1;
    kvs::TransferFunction tfunc( 256 );
    const auto ntype = normal_type == 0 ? kvs::PolygonObject::PolygonNormal : kvs::PolygonObject::VertexNormal;
    auto* vol = new kvs::StructuredVolumeObject();
    vol->setVeclen( 1 );
    vol->setResolution( kvs::Vec3ui( nx, ny, nz ) );
    vol->setValues( vals );
    vol->setGridTypeToUniform();
    auto* mc = new kvs::MarchingCubes( vol, isolevel, ntype, duplication != 0, tfunc );
    int rc = -2;
    if ( format <= 1 )
    {
        kvs::PolygonExporter<kvs::Stl> exporter( mc );
        if ( exporter.kvs::ExporterBase::isSuccess() )
        {
            exporter.setFileType( format == 0 ? kvs::Stl::Binary : kvs::Stl::Ascii );
            rc = exporter.write( path ) ? 0 : -3;
        }
    }
    else
    {
        kvs::PolygonExporter<kvs::KVSMLPolygonObject> exporter( mc );
        if ( exporter.kvs::ExporterBase::isSuccess() )
        {
            if ( format == 2 ) exporter.setWritingDataTypeToAscii();
            else if ( format == 3 ) exporter.setWritingDataTypeToExternalAscii();
            else exporter.setWritingDataTypeToExternalBinary();
            rc = exporter.write( path ) ? 0 : -3;
        }
    }
    delete mc;
    delete vol;
    return rc;
}

/*
 * kvs::PolygonExporter<kvs::Ply> (PolygonExporter.cpp:178-361) + Ply::write
 * with the Binary file type (Ply.cpp:389-488) of a PolygonObject built from
 * raw arrays: coords (3 per vertex), colors (ncolors bytes: 3 = one colour),
 * normals, connections (may be empty), color_type / normal_type as
 * kvs::PolygonObject's enums (0 vertex, 1 polygon).  Returns 0 when written,
 * -2 when the exporter failed.
 */
int kvsref_write_ply( const float* coords, unsigned long long ncoords, const unsigned char* colors,
                      unsigned long long ncolors, const float* normals, unsigned long long nnormals,
                      int color_type, int normal_type, const char* path )
{
    kvs::PolygonObject poly;
    poly.setPolygonType( kvs::PolygonObject::Triangle );
    poly.setColorType( color_type == 0 ? kvs::PolygonObject::VertexColor : kvs::PolygonObject::PolygonColor );
    poly.setNormalType( normal_type == 0 ? kvs::PolygonObject::VertexNormal : kvs::PolygonObject::PolygonNormal );
    poly.setCoords( kvs::ValueArray<kvs::Real32>( coords, ncoords ) );
    if ( ncolors ) poly.setColors( kvs::ValueArray<kvs::UInt8>( colors, ncolors ) );
    if ( nnormals ) poly.setNormals( kvs::ValueArray<kvs::Real32>( normals, nnormals ) );
    kvs::PolygonExporter<kvs::Ply> exporter( &poly );
    if ( !exporter.kvs::ExporterBase::isSuccess() ) return -2;
    exporter.setFileType( kvs::Ply::Binary );
    return exporter.write( path ) ? 0 : -3;
}

/*
 * The reference kvs::Isosurface (Source/Core/Visualization/Mapper/Isosurface.cpp)
 * on a uniform structured volume, through one of its three constructors:
 *   form 0: Isosurface( volume, normal_type )   -- isolevel = (max + min) * 0.5
 *   form 1: Isosurface( volume, isolevel, normal_type )
 *   form 2: Isosurface( volume, isolevel, normal_type, duplication, tfunc )
 */
int kvsref_isosurface(
    int form, int dtype, const void* values, unsigned nx, unsigned ny, unsigned nz,
    double isolevel, int normal_type, int duplication, int has_minmax, double vmin, double vmax,
    int tf_resolution, int tf_has_range, float tf_min, float tf_max, kvsref_result* out )
{
    std::memset( out, 0, sizeof( *out ) );
    const size_t n = size_t( nx ) * ny * nz;
    kvs::AnyValueArray vals = Values( dtype, values, n );
    if ( vals.size() != n ) return -1;
    kvs::TransferFunction tfunc( tf_resolution > 0 ? tf_resolution : 256 );
    if ( tf_has_range ) tfunc.setRange( tf_min, tf_max );
    const auto ntype = normal_type == 0 ? kvs::PolygonObject::PolygonNormal : kvs::PolygonObject::VertexNormal;
    auto* vol = new kvs::StructuredVolumeObject();
    vol->setVeclen( 1 );
    vol->setResolution( kvs::Vec3ui( nx, ny, nz ) );
    vol->setValues( vals );
    vol->setGridTypeToUniform();
    if ( has_minmax ) vol->setMinMaxValues( vmin, vmax );
    kvs::Isosurface* iso = nullptr;
    if ( form == 0 ) iso = new kvs::Isosurface( vol, ntype );
    else if ( form == 1 ) iso = new kvs::Isosurface( vol, isolevel, ntype );
    else iso = new kvs::Isosurface( vol, isolevel, ntype, duplication != 0, tfunc );
    Fill( iso, iso, vol, out );
    delete iso;
    delete vol;
    return 0;
}

void kvsref_free( kvsref_result* r )
{
    std::free( r->coords );
    std::free( r->normals );
    std::free( r->connections );
    std::free( r->colors );
    std::free( r->opacities );
    std::memset( r, 0, sizeof( *r ) );
}

/*
 * The unstructured marching mappers (MarchingTetrahedra, MarchingHexahedra,
 * MarchingPyramid, MarchingPrism) on an UnstructuredVolumeObject built from
 * raw arrays.  cell_type: 0 tetrahedra, 1 hexahedra, 2 pyramid, 3 prism.
 * form 0: the cell type's mapper (volume, isolevel, normal_type, duplication,
 * tfunc); form 1: Isosurface( volume, isolevel, normal_type, duplication,
 * tfunc ), which routes by cell type (Isosurface.cpp:193-258).
 * repeat: run this many times on fresh volumes, report the fastest.
 */
int kvsref_marching_cells(
    int form, int cell_type, int dtype, const void* values, unsigned long long nnodes, const float* coords,
    const unsigned int* connections, unsigned long long ncells, double isolevel, int normal_type,
    int duplication, int has_minmax, double vmin, double vmax, int tf_resolution, int tf_has_range,
    float tf_min, float tf_max, int repeat, kvsref_result* out )
{
    std::memset( out, 0, sizeof( *out ) );
    static const kvs::UnstructuredVolumeObject::CellType types[4] = {
        kvs::UnstructuredVolumeObject::Tetrahedra, kvs::UnstructuredVolumeObject::Hexahedra,
        kvs::UnstructuredVolumeObject::Pyramid, kvs::UnstructuredVolumeObject::Prism };
    static const size_t npc[4] = { 4, 8, 5, 6 };
    if ( cell_type < 0 || cell_type > 3 ) return -1;
    kvs::AnyValueArray vals = Values( dtype, values, nnodes );
    if ( vals.size() != nnodes ) return -1;
    kvs::TransferFunction tfunc( tf_resolution > 0 ? tf_resolution : 256 );
    if ( tf_has_range ) tfunc.setRange( tf_min, tf_max );
    const auto ntype = normal_type == 0 ? kvs::PolygonObject::PolygonNormal : kvs::PolygonObject::VertexNormal;
    double best = 1e300;
    for ( int r = 0; r < ( repeat > 0 ? repeat : 1 ); ++r )
    {
        auto* vol = new kvs::UnstructuredVolumeObject();
        vol->setCellType( types[cell_type] );
        vol->setVeclen( 1 );
        vol->setNumberOfNodes( nnodes );
        vol->setNumberOfCells( ncells );
        vol->setCoords( kvs::ValueArray<kvs::Real32>( coords, 3 * nnodes ) );
        vol->setConnections( kvs::ValueArray<kvs::UInt32>( connections, npc[cell_type] * ncells ) );
        vol->setValues( vals );
        if ( has_minmax ) vol->setMinMaxValues( vmin, vmax );
        const auto t0 = std::chrono::steady_clock::now();
        kvs::PolygonObject* poly = nullptr;
        kvs::MapperBase* mapper = nullptr;
        if ( form == 1 )
        {
            auto* m = new kvs::Isosurface( vol, isolevel, ntype, duplication != 0, tfunc );
            poly = m; mapper = m;
        }
        else if ( cell_type == 0 )
        {
            auto* m = new kvs::MarchingTetrahedra( vol, isolevel, ntype, duplication != 0, tfunc );
            poly = m; mapper = m;
        }
        else if ( cell_type == 1 )
        {
            auto* m = new kvs::MarchingHexahedra( vol, isolevel, ntype, duplication != 0, tfunc );
            poly = m; mapper = m;
        }
        else if ( cell_type == 2 )
        {
            auto* m = new kvs::MarchingPyramid( vol, isolevel, ntype, duplication != 0, tfunc );
            poly = m; mapper = m;
        }
        else
        {
            auto* m = new kvs::MarchingPrism( vol, isolevel, ntype, duplication != 0, tfunc );
            poly = m; mapper = m;
        }
        const double dt = std::chrono::duration<double>( std::chrono::steady_clock::now() - t0 ).count();
        if ( dt < best ) best = dt;
        if ( r + 1 == ( repeat > 0 ? repeat : 1 ) )
        {
            kvsref_free( out );
            Fill( mapper, poly, vol, out );
            out->seconds = best;
        }
        delete poly;
        delete vol;
    }
    return 0;
}

/* HydrogenVolumeData (Source/Core/Visualization/Data/HydrogenVolumeData.cpp):
 * the reference's own deterministic uint8 field, res^3 nodes. */
int kvsref_hydrogen( unsigned res, unsigned char* out )
{
    kvs::HydrogenVolumeData h( kvs::Vec3ui( res, res, res ) );
    h.exec();
    const auto& v = h.values();
    if ( v.size() != size_t( res ) * res * res ) return -1;
    std::memcpy( out, v.data(), v.size() );
    return 0;
}

/* The transfer function's colour table (resolution x RGB) and ColorMap::at
 * for the default map, so the host-side colour can be pinned too. */
int kvsref_default_colormap( int resolution, unsigned char* table )
{
    kvs::TransferFunction tf( resolution );
    const auto& t = tf.colorMap().table();
    std::memcpy( table, t.data(), t.size() );
    return int( t.size() );
}

int kvsref_color_at( int resolution, float tf_min, float tf_max, float value, unsigned char* rgb )
{
    kvs::TransferFunction tf( resolution );
    tf.setRange( tf_min, tf_max );
    const kvs::RGBColor c = tf.colorMap().at( value );
    rgb[0] = c.r(); rgb[1] = c.g(); rgb[2] = c.b();
    return 0;
}

} // extern "C"
