/*****************************************************************************/
/**
 *  @file   Isosurface.cpp
 *  @brief  kvs::cuda::Isosurface on kvs::cuda::MarchingCubes.
 *
 *  The flow is the reference's (Source/Core/Visualization/Mapper/Isosurface.cpp):
 *  the constructors (:23-96) set the normal type, take the default isolevel
 *  (max + min) * 0.5 from the volume's min/max cache and make VertexNormal
 *  imply shared vertices; exec (:104-124) checks the input; mapping
 *  (:132-258) builds the per-grid mapper and shallow-copies its arrays.
 *  What changes: the structured branch's mapper is kvs::cuda::MarchingCubes,
 *  the unstructured branch's are kvs::cuda::MarchingTetrahedra / Hexahedra /
 *  Pyramid / Prism, the min/max scan behind the default isolevel runs on the
 *  GPU, and a GPU failure is reported and ends exec with nullptr instead of
 *  leaving empty arrays behind.  As in the reference, this mapper never sets isSuccess()
 *  true (MapperBase's initial false, MapperBase.cpp:23).
 */
/*****************************************************************************/
#include "Isosurface.h"

#include <kvs/Message>
#include <kvs/StructuredVolumeObject>
#include <kvs/UnstructuredVolumeObject>

#include <limits>

#include "Context.h"
#include "MarchingCells.h"
#include "MarchingCubes.h"

namespace
{

// StructuredVolumeObject::updateMinMaxValues (StructuredVolumeObject.cpp:431-450)
// by the device scan (GetMinMaxValues' rules); the cache is mutable in the
// reference too (VolumeObjectBase.h:51-53).
bool DeviceMinMax( const kvs::StructuredVolumeObject* volume, int device )
{
    const int dtype = kvs::cuda::DType( volume->values() );
    if ( dtype < 0 ) return false;
    kvsmc_status st = KVSMC_OK;
    kvsmc_context* ctx = kvs::cuda::DeviceContext( device, &st );
    if ( !ctx )
    {
        kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
        return false;
    }
    const auto res = volume->resolution();
    kvsmc_volume* v = nullptr;
    double mn = 0, mx = 0;
    st = kvsmc_volume_upload( ctx, volume->values().data(), kvsmc_dtype( dtype ), res.x(), res.y(), res.z(), &v );
    if ( st == KVSMC_OK ) st = kvsmc_volume_minmax( ctx, v, &mn, &mx );
    if ( v ) kvsmc_volume_free( ctx, v );
    if ( st != KVSMC_OK )
    {
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }
    volume->setMinMaxValues( mn, mx );
    return true;
}

// UnstructuredVolumeObject::updateMinMaxValues (UnstructuredVolumeObject.cpp:469-487)
// by the device scan over values[0] and the cells' nodes: a marching call at
// isolevel NaN, where no node is above, so only the scan and an empty count
// pass run.
bool DeviceMinMax( const kvs::UnstructuredVolumeObject* volume, int device )
{
    int cell = -1;
    switch ( volume->cellType() )
    {
    case kvs::UnstructuredVolumeObject::Tetrahedra: cell = KVSMC_TETRAHEDRA; break;
    case kvs::UnstructuredVolumeObject::Hexahedra: cell = KVSMC_HEXAHEDRA; break;
    case kvs::UnstructuredVolumeObject::Pyramid: cell = KVSMC_PYRAMID; break;
    case kvs::UnstructuredVolumeObject::Prism: cell = KVSMC_PRISM; break;
    default: break;
    }
    const int dtype = kvs::cuda::DType( volume->values() );
    if ( cell < 0 || dtype < 0 || volume->veclen() != 1 )
    {
        volume->updateMinMaxValues();   // what no marching mapper takes: the reference's own scan
        return true;
    }
    kvsmc_status st = KVSMC_OK;
    kvsmc_context* ctx = kvs::cuda::DeviceContext( device, &st );
    if ( !ctx )
    {
        kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
        return false;
    }
    kvsmc_sizes sizes{};
    st = kvsmc_marching_cells_host( ctx, kvsmc_cell_type( cell ), volume->values().data(), kvsmc_dtype( dtype ),
                                    volume->numberOfNodes(), volume->coords().data(), volume->connections().data(),
                                    volume->numberOfCells(), std::numeric_limits<double>::quiet_NaN(), 0, 0.0, 0.0,
                                    []( void*, int32_t, uint64_t ) -> void* { return nullptr; }, nullptr, &sizes );
    if ( st != KVSMC_OK )
    {
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }
    volume->setMinMaxValues( sizes.min_value, sizes.max_value );
    return true;
}

} // end of namespace

namespace kvs
{

namespace cuda
{

Isosurface::Isosurface(
    const kvs::VolumeObjectBase* volume,
    const SuperClass::NormalType normal_type ):
    kvs::MapperBase(),
    kvs::PolygonObject()
{
    SuperClass::setNormalType( normal_type );
    if ( !volume->hasMinMaxValues() )
    {
        const auto* svolume = kvs::StructuredVolumeObject::DownCast( volume );
        const auto* uvolume = kvs::UnstructuredVolumeObject::DownCast( volume );
        if ( svolume ) { if ( !DeviceMinMax( svolume, m_device ) ) return; }
        else if ( uvolume ) { if ( !DeviceMinMax( uvolume, m_device ) ) return; }
        else { volume->updateMinMaxValues(); }
    }
    this->setIsolevel( ( volume->maxValue() + volume->minValue() ) * 0.5 );
    if ( normal_type == kvs::PolygonObject::VertexNormal ) { m_duplication = false; }
    this->exec( volume );
}

Isosurface::Isosurface(
    const kvs::VolumeObjectBase* volume,
    const double isolevel,
    const NormalType normal_type ):
    kvs::MapperBase(),
    kvs::PolygonObject(),
    m_isolevel( isolevel )
{
    SuperClass::setNormalType( normal_type );
    if ( normal_type == kvs::PolygonObject::VertexNormal ) { m_duplication = false; }
    this->exec( volume );
}

Isosurface::Isosurface(
    const kvs::VolumeObjectBase* volume,
    const double isolevel,
    const NormalType normal_type,
    const bool duplication,
    const kvs::TransferFunction& transfer_function ):
    kvs::MapperBase( transfer_function ),
    kvs::PolygonObject(),
    m_isolevel( isolevel ),
    m_duplication( duplication )
{
    SuperClass::setNormalType( normal_type );
    if ( normal_type == kvs::PolygonObject::VertexNormal ) { m_duplication = false; }
    this->exec( volume );
}

Isosurface::SuperClass* Isosurface::exec( const kvs::ObjectBase* object )
{
    if ( !object )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is NULL.");
        return nullptr;
    }

    const auto* volume = kvs::VolumeObjectBase::DownCast( object );
    if ( !volume )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is not volume dat.");
        return nullptr;
    }

    if ( !this->mapping( volume ) ) { return nullptr; }
    return this;
}

void Isosurface::shallowCopy( const kvs::PolygonObject* polygon )
{
    SuperClass::setCoords( polygon->coords() );
    SuperClass::setColors( polygon->colors() );
    SuperClass::setNormals( polygon->normals() );
    SuperClass::setConnections( polygon->connections() );
    SuperClass::setOpacities( polygon->opacities() );
    SuperClass::setPolygonType( polygon->polygonType() );
    SuperClass::setColorType( polygon->colorType() );
    SuperClass::setNormalType( polygon->normalType() );
    SuperClass::setMinMaxObjectCoords( polygon->minObjectCoord(), polygon->maxObjectCoord() );
    SuperClass::setMinMaxExternalCoords( polygon->minExternalCoord(), polygon->maxExternalCoord() );
}

bool Isosurface::mapping( const kvs::VolumeObjectBase* volume )
{
    if ( volume->veclen() != 1 )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is not scalar field dat.");
        return true;   // the reference returns `this` here
    }

    const auto ntype = SuperClass::normalType();
    const auto tfunc = BaseClass::transferFunction();

    if ( volume->volumeType() == kvs::VolumeObjectBase::Structured )
    {
        const auto* svolume = kvs::StructuredVolumeObject::DownCast( volume );
        kvs::cuda::MarchingCubes polygon;
        polygon.setDevice( m_device );
        polygon.setNormalType( ntype );
        polygon.setTransferFunction( tfunc );
        polygon.setDuplication( m_duplication );
        polygon.setIsolevel( m_isolevel );
        if ( !polygon.exec( svolume ) )
        {
            BaseClass::setSuccess( false );
            kvsMessageError("Cannot create isosurfaces.");
            return false;
        }
        this->shallowCopy( &polygon );
        return true;
    }

    // unstructured grids (Isosurface.cpp:193-258)
    const auto* uvolume = kvs::UnstructuredVolumeObject::DownCast( volume );
    kvs::cuda::MarchingCellsBase* polygon = nullptr;
    kvs::cuda::MarchingTetrahedra tet;
    kvs::cuda::MarchingHexahedra hex;
    kvs::cuda::MarchingPyramid pyr;
    kvs::cuda::MarchingPrism pri;
    kvs::PolygonObject* result = nullptr;
    switch ( uvolume->cellType() )
    {
    case kvs::UnstructuredVolumeObject::Tetrahedra: polygon = &tet; break;
    case kvs::UnstructuredVolumeObject::Hexahedra: polygon = &hex; break;
    case kvs::UnstructuredVolumeObject::Pyramid: polygon = &pyr; break;
    case kvs::UnstructuredVolumeObject::Prism: polygon = &pri; break;
    default: return true;   // no mapper: empty arrays, as in the reference
    }
    polygon->setDevice( m_device );
    polygon->setNormalType( ntype );
    polygon->setTransferFunction( tfunc );
    polygon->setDuplication( m_duplication );
    polygon->setIsolevel( m_isolevel );
    if ( polygon == &tet ) result = tet.exec( uvolume );
    else if ( polygon == &hex ) result = hex.exec( uvolume );
    else if ( polygon == &pyr ) result = pyr.exec( uvolume );
    else result = pri.exec( uvolume );
    if ( !result )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Cannot create isosurfaces.");
        return false;
    }
    this->shallowCopy( polygon );
    return true;
}

} // end of namespace cuda

} // end of namespace kvs
