/*****************************************************************************/
/**
 *  @file   MarchingCubes.cpp
 *  @brief  kvs::cuda::MarchingCubes on libkvsmc.
 *
 *  The flow is the reference's (Source/Core/Visualization/Mapper/MarchingCubes.cpp):
 *  exec (:46-79) validates the input and makes VertexNormal imply shared
 *  vertices; mapping (:87-132) attaches the volume, fixes the bounding box,
 *  the polygon/normal/colour types, and runs the extraction.  What changes:
 *  the min/max scan and everything per cell run on the GPU in one C call
 *  (kvsmc_marching_cubes_host), and the output arrays are allocated as
 *  kvs::ValueArray by that call's allocator, so no vector->ValueArray copy
 *  is made (the reference copies, :236-242).
 */
/*****************************************************************************/
#include "MarchingCubes.h"

#include <map>

#include <kvs/Message>
#include <kvs/ValueArray>

#include "Context.h"
#include "kvsmc.h"

namespace
{

// One libkvsmc context per (host thread, device), kept for the thread's life:
// mapper objects are short-lived (kvs::Isosurface makes one per call), the
// context's stream and arenas are not.
struct ContextCache
{
    std::map<int, kvsmc_context*> contexts;
    ~ContextCache() { for ( auto& c : contexts ) kvsmc_destroy( c.second ); }
};

kvsmc_context* Context( int device, kvsmc_status* status )
{
    thread_local ContextCache cache;
    auto it = cache.contexts.find( device );
    if ( it != cache.contexts.end() ) { *status = KVSMC_OK; return it->second; }
    kvsmc_context* ctx = nullptr;
    *status = kvsmc_create( device, &ctx );
    if ( *status != KVSMC_OK ) return nullptr;
    cache.contexts[ device ] = ctx;
    return ctx;
}

} // end of namespace

namespace kvs
{
namespace cuda
{

kvsmc_context* DeviceContext( int device, kvsmc_status* status ) { return Context( device, status ); }

// kvs::Type::TypeID -> kvsmc_dtype (the reference's type switch, :113-124)
int DType( const kvs::AnyValueArray& values )
{
    switch ( values.typeID() )
    {
    case kvs::Type::TypeInt8: return KVSMC_I8;
    case kvs::Type::TypeInt16: return KVSMC_I16;
    case kvs::Type::TypeInt32: return KVSMC_I32;
    case kvs::Type::TypeInt64: return KVSMC_I64;
    case kvs::Type::TypeUInt8: return KVSMC_U8;
    case kvs::Type::TypeUInt16: return KVSMC_U16;
    case kvs::Type::TypeUInt32: return KVSMC_U32;
    case kvs::Type::TypeUInt64: return KVSMC_U64;
    case kvs::Type::TypeReal32: return KVSMC_F32;
    case kvs::Type::TypeReal64: return KVSMC_F64;
    default: return -1;
    }
}

} // end of namespace cuda
} // end of namespace kvs

namespace
{

using kvs::cuda::DType;

// The arrays the C call asks for, allocated as the PolygonObject's own.
struct Outputs
{
    kvs::ValueArray<kvs::Real32> coords;
    kvs::ValueArray<kvs::Real32> normals;
    kvs::ValueArray<kvs::UInt32> connections;
};

void* Allocate( void* user, int32_t which, uint64_t count )
{
    Outputs* o = static_cast<Outputs*>( user );
    switch ( which )
    {
    case 0: o->coords.allocate( count ); return o->coords.data();
    case 1: o->normals.allocate( count ); return o->normals.data();
    case 2: o->connections.allocate( count ); return o->connections.data();
    default: return nullptr;
    }
}

} // end of namespace

namespace kvs
{

namespace cuda
{

MarchingCubes::MarchingCubes(
    const kvs::StructuredVolumeObject* volume,
    const double isolevel,
    const NormalType normal_type,
    const bool duplication,
    const kvs::TransferFunction& transfer_function ):
    kvs::MapperBase( transfer_function ),
    m_isolevel( isolevel ),
    m_duplication( duplication )
{
    SuperClass::setNormalType( normal_type );
    this->exec( volume );
}

MarchingCubes::SuperClass* MarchingCubes::exec( const kvs::ObjectBase* object )
{
    BaseClass::setSuccess( false );

    if ( !object )
    {
        kvsMessageError("Input object is NULL.");
        return nullptr;
    }

    const auto* volume = kvs::StructuredVolumeObject::DownCast( object );
    if ( !volume )
    {
        kvsMessageError("Input object is not structured volume object.");
        return nullptr;
    }

    if ( volume->veclen() != 1 )
    {
        kvsMessageError("Input volume is not sclar field data.");
        return nullptr;
    }

    // VertexNormal forces shared vertices, and it sticks (MarchingCubes.cpp:69-73).
    if ( SuperClass::normalType() == kvs::PolygonObject::VertexNormal )
    {
        m_duplication = false;
    }

    if ( !this->mapping( volume ) ) { return nullptr; }

    BaseClass::setSuccess( true );
    return this;
}

bool MarchingCubes::mapping( const kvs::StructuredVolumeObject* volume )
{
    BaseClass::attachVolume( volume );
    BaseClass::setMinMaxCoords( volume, this );

    SuperClass::setPolygonTypeToTriangle();
    if ( m_duplication ) SuperClass::setNormalTypeToPolygon();
    SuperClass::setColorTypeToPolygon();

    const int dtype = DType( volume->values() );
    if ( dtype < 0 )
    {
        kvsMessageError("Unsupported data type '%s'.", volume->values().typeInfo()->typeName() );
        return true;   // the reference reports and still returns success
    }

    kvsmc_params p;
    p.isolevel = m_isolevel;
    p.mode = ( SuperClass::normalType() == kvs::PolygonObject::VertexNormal ) ? KVSMC_SHARED_VERTEX_NORMAL
           : ( m_duplication ? KVSMC_DUP_POLYGON_NORMAL : KVSMC_SHARED_POLYGON_NORMAL );
    p.has_minmax = volume->hasMinMaxValues() ? 1 : 0;
    p.min_value = volume->minValue();
    p.max_value = volume->maxValue();
    const auto ncells = volume->resolution() - kvs::Vec3u::Constant(1);
    const auto min_coord = volume->minObjectCoord();
    const auto max_coord = volume->maxObjectCoord();
    const auto scale_factor = ( max_coord - min_coord ) / kvs::Vec3{ ncells };   // MarchingCubes.cpp:166-168
    for ( int k = 0; k < 3; ++k ) { p.min_coord[k] = min_coord[k]; p.scale[k] = scale_factor[k]; }

    kvsmc_status st = KVSMC_OK;
    kvsmc_context* ctx = Context( m_device, &st );
    if ( !ctx )
    {
        kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
        return false;
    }
    Outputs out;
    kvsmc_sizes sizes;
    const auto res = volume->resolution();
    st = kvsmc_marching_cubes_host( ctx, volume->values().data(), kvsmc_dtype( dtype ), res.x(), res.y(), res.z(),
                                    &p, &Allocate, &out, &sizes );
    if ( st != KVSMC_OK )
    {
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }

    // MapperBase::setRange (MapperBase.cpp:54-83): the volume's min/max cache
    // (filled here by the device scan), then the transfer function's range.
    if ( !volume->hasMinMaxValues() ) volume->setMinMaxValues( sizes.min_value, sizes.max_value );
    BaseClass::setRange( volume );

    if ( !sizes.extracted ) return true;   // Math::Equal(min, max): MarchingCubes.cpp:108-110
    if ( out.coords.size() > 0 )
    {
        SuperClass::setCoords( out.coords );
        if ( !m_duplication ) SuperClass::setConnections( out.connections );
        SuperClass::setColor( BaseClass::transferFunction().colorMap().at( m_isolevel ) );
        SuperClass::setNormals( out.normals );
        SuperClass::setOpacity( 255 );
    }
    return true;
}

} // end of namespace cuda

} // end of namespace kvs
