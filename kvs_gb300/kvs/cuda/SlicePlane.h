/*****************************************************************************/
/**
 *  @file   SlicePlane.h
 *  @brief  kvs::cuda::SlicePlane -- kvs::SlicePlane with its structured-grid
 *          branch on the GPU.
 *
 *  Same constructors, setPlane and exec(ObjectBase*) as the reference mapper
 *  (Source/Core/Visualization/Mapper/SlicePlane.h:25-79); a structured
 *  volume is sliced by libkvsmc (kvsmc_slice_plane) with the same
 *  PolygonObject bits, and so is an unstructured volume of tetrahedra,
 *  hexahedra, pyramids or prisms (kvsmc_slice_cells_host).  When the GPU call fails, exec reports
 *  kvsMessageError and returns nullptr (no CPU fallback).
 */
/*****************************************************************************/
#pragma once
#include <kvs/MapperBase>
#include <kvs/Module>
#include <kvs/PolygonObject>
#include <kvs/UnstructuredVolumeObject>
#include <kvs/VolumeObjectBase>
#include <kvs/Vector3>
#include <kvs/Vector4>

namespace kvs
{

namespace cuda
{

class SlicePlane : public kvs::MapperBase, public kvs::PolygonObject
{
    kvsModule( kvs::cuda::SlicePlane, Mapper );
    kvsModuleBaseClass( kvs::MapperBase );
    kvsModuleSuperClass( kvs::PolygonObject );

private:
    kvs::Vec4 m_coef{ 0.0f, 0.0f, 0.0f, 0.0f }; ///< coefficients of the slice plane
    int m_device = -1;                           ///< CUDA device (-1: the current one)

public:
    SlicePlane() = default;
    virtual ~SlicePlane() = default;

    SlicePlane(
        const kvs::VolumeObjectBase* volume,
        const kvs::Vec4& coefficients,
        const kvs::TransferFunction& transfer_function );
    SlicePlane(
        const kvs::VolumeObjectBase* volume,
        const kvs::Vec3& point,
        const kvs::Vec3& normal,
        const kvs::TransferFunction& transfer_function );

    void setPlane( const kvs::Vec4& coef ) { m_coef = coef; }
    void setPlane( const kvs::Vec3& point, const kvs::Vec3& normal ) { m_coef = { normal, -point.dot( normal ) }; }
    void setDevice( const int device ) { m_device = device; }

    SuperClass* exec( const kvs::ObjectBase* object );

private:
    bool mapping( const kvs::VolumeObjectBase* volume );
    bool mapping_cells( const kvs::UnstructuredVolumeObject* volume );
};

} // end of namespace cuda

} // end of namespace kvs
