"""
    FlexShellGPU

Julia-side binding of libflexshell.so (include/flexshell.h).  It adds methods
with the reference signatures of FinEtoolsFlexStructures.jl 3.6.4 so that
driver code calls them unchanged:

    stiffness(femm::FEMMShellT3FF, assembler, geom0, u1, Rfield1, dchi)
    mass(femm::FEMMShellT3FF, assembler, geom0, dchi)

(and the same for FEMMShellQ4RS, FEMMShellT3FFComp, FEMMShellQ4RSComp),

    inspectintegpoints(femm, geom0, u, dT, felist, inspector, idat, quantity; outputcsys)

for FEMMShellT3FF and FEMMShellQ4RS, and for FEMMCorotBeam

    stiffness / geostiffness (femm, assembler, geom0, u1, Rfield1, dchi)
    mass(femm, assembler, geom0, u1, Rfield1, dchi; mass_type)
    gyroscopic(femm, assembler, geom0, u1, Rfield1, v1, dchi; mass_type)
    restoringforce(femm, assembler, geom0, u1, Rfield1, dchi)
    distribloads_global(femm, assembler, geom0, u1, Rfield1, dchi, fi)

and, for the distributed loads on a shell element set,

    gpu_distribloads(femm::FEMMBase, assembler, geom, P, fi, m)

`associategeometry!` stays the reference's own; its normals are passed in.
Not exercised in this repository (no Julia toolchain here); it is the
binding a maintainer adds next to the reference.
"""
module FlexShellGPU

using SparseArrays
using FinEtools
using FinEtoolsFlexStructures.FEMMShellT3FFModule: FEMMShellT3FF
using FinEtoolsFlexStructures.FEMMShellQ4RSModule: FEMMShellQ4RS
import FinEtoolsFlexStructures.FEMMShellT3FFModule: stiffness, mass
import FinEtoolsFlexStructures.FEMMShellQ4RSModule: stiffness, mass
import FinEtoolsFlexStructures.FEMMShellT3FFModule: inspectintegpoints
import FinEtoolsFlexStructures.FEMMShellQ4RSModule: inspectintegpoints
using FinEtoolsFlexStructures.FEMMCorotBeamModule: FEMMCorotBeam
import FinEtoolsFlexStructures.FEMMCorotBeamModule: geostiffness, gyroscopic, restoringforce,
    distribloads_global

const libflexshell = get(ENV, "FLEXSHELL_LIB", "libflexshell.so")

const FS_T3FF, FS_T3FFCOMP, FS_Q4RS, FS_Q4RSCOMP, FS_COROTBEAM = 0, 1, 2, 3, 4
const FS_BEAM_STIFFNESS, FS_BEAM_GEOSTIFFNESS, FS_BEAM_MASS, FS_BEAM_GYROSCOPIC = 0, 1, 2, 3
const FS_FP64, FS_MIXED = 0, 1
const FS_ASM_SPARSE, FS_ASM_SPARSE_SYMM, FS_ASM_DIAG = 0, 1, 2

# fs_shell_params (include/flexshell.h)
struct FsShellParams
    transv_shear_formulation::Int32
    reserved::Int32
    drilling_stiffness_scale::Float64
    threshold_angle::Float64
    stab_c::Float64
    Dps::NTuple{9,Float64}
    Dt::NTuple{4,Float64}
    rho::Float64
    thickness::Float64
end

mutable struct Ctx
    h::Ptr{Cvoid}
end

function check(ctx::Ctx, st::Cint)
    st == 0 && return nothing
    buf = Vector{UInt8}(undef, 512)
    ccall((:fs_last_error, libflexshell), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), ctx.h, buf, 512)
    msg = unsafe_string(pointer(buf))
    st == 6 && throw(AssertionError(msg))       # FS_ERR_STATE: the reference @assert
    throw(ErrorException("flexshell error $st: $msg"))
end

const CONTEXTS = IdDict{Any,Ctx}()

function context(femm)
    get!(CONTEXTS, femm) do
        r = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:fs_ctx_create, libflexshell), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, r)
        st == 0 || error("flexshell: no CUDA device")
        ctx = Ctx(r[])
        finalizer(c -> ccall((:fs_ctx_destroy, libflexshell), Cint, (Ptr{Cvoid},), c.h), ctx)
        ctx
    end
end

# stab_fun restricted to t^2/(t^2 + c h^2): recover c, verify at two points
function stab_coefficient(f)
    c = 1 / f(1.0, 1.0) - 1
    for (t, h) in ((0.3, 2.0), (0.01, 0.05))
        isapprox(f(t, h), t^2 / (t^2 + c * h^2); rtol = 1e-12) ||
            throw(ArgumentError("stab_fun is not of the form t^2/(t^2 + c h^2)"))
    end
    return c
end

asm_mode(::SysmatAssemblerSparseSymm) = FS_ASM_SPARSE_SYMM
asm_mode(::SysmatAssemblerSparseDiag) = FS_ASM_DIAG
asm_mode(::AbstractSysmatAssembler) = FS_ASM_SPARSE

function upload!(ctx, femm, etype, geom0, dchi)
    fes = femm.integdomain.fes
    conn = collect(reinterpret(Int, fes.conn))          # nen per element, 1-based
    xyz = geom0.values                                  # nnodes x 3, column-major
    check(ctx, ccall((:fs_mesh_set, libflexshell), Cint,
        (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}),
        ctx.h, etype, size(xyz, 1), xyz, count(fes), conn, C_NULL, dchi === nothing ? C_NULL : dchi.dofnums))
    Dps, Dt = femm_material_matrices(femm)
    t = femm.integdomain.otherdimension(zeros(1, 3), fes.conn[1], zeros(1, 1))
    p = FsShellParams(etype == FS_T3FF ? femm.transv_shear_formulation : 0, 0,
        femm.drilling_stiffness_scale, femm.threshold_angle, stab_coefficient(femm.stab_fun),
        Tuple(vec(Dps)), Tuple(vec(Dt)), massdensity(femm.material), t)
    check(ctx, ccall((:fs_params_set, libflexshell), Cint, (Ptr{Cvoid}, Ref{FsShellParams}, Ptr{Float64}),
        ctx.h, p, C_NULL))
    # normals from the reference's associategeometry! (honours a user mcsys)
    check(ctx, ccall((:fs_normals_set, libflexshell), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{UInt8}),
        ctx.h, femm._normals, UInt8.(femm._normal_valid)))
end

femm_material_matrices(femm) =
    FinEtoolsFlexStructures.FEMMShellT3FFModule._shell_material_stiffness(femm.material)

function fetch_csc(ctx, n, nnz)
    colptr = Vector{Int64}(undef, n + 1)
    rowval = Vector{Int64}(undef, nnz)
    nzval = Vector{Float64}(undef, nnz)
    check(ctx, ccall((:fs_matrix_copy, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}), ctx.h, colptr, rowval, nzval))
    return SparseMatrixCSC(n, n, colptr, rowval, nzval)
end

for (T, etype) in ((FEMMShellT3FF, FS_T3FF), (FEMMShellQ4RS, FS_Q4RS))
    @eval function stiffness(self::$T, assembler::ASS, geom0::NodalField{Float64},
        u1::NodalField{TI}, Rfield1::NodalField{TI}, dchi::NodalField{TI};
        precision = FS_FP64) where {ASS<:AbstractSysmatAssembler,TI<:Number}
        @assert self._associatedgeometry == true
        ctx = context(self)
        upload!(ctx, self, $etype, geom0, dchi)
        nnz = Ref{Int64}(0)
        check(ctx, ccall((:fs_stiffness, libflexshell), Cint, (Ptr{Cvoid}, Cint, Cint, Int64, Ref{Int64}),
            ctx.h, precision, asm_mode(assembler), nalldofs(dchi), nnz))
        return fetch_csc(ctx, nalldofs(dchi), nnz[])
    end
    @eval function mass(self::$T, assembler::A, geom0::NodalField{Float64},
        dchi::NodalField{TI}) where {A<:AbstractSysmatAssembler,TI<:Number}
        @assert self._associatedgeometry == true
        ctx = context(self)
        upload!(ctx, self, $etype, geom0, dchi)
        nnz = Ref{Int64}(0)
        check(ctx, ccall((:fs_mass, libflexshell), Cint, (Ptr{Cvoid}, Cint, Int64, Ref{Int64}),
            ctx.h, asm_mode(assembler), nalldofs(dchi), nnz))
        return fetch_csc(ctx, nalldofs(dchi), nnz[])
    end
end

# ---------------------------------------------------------------------------
# inspectintegpoints (src/FEMMShellT3FFModule.jl:850-962,
# src/FEMMShellQ4RSModule.jl:1061-1170): the resultants of every integration
# point come from one fs_resultants call; the output csys is evaluated here,
# per point, with the reference's own updatecsmat!, and the inspector is then
# called for the points of felist in the reference's order.
# ---------------------------------------------------------------------------
const FS_RES_MOMENT, FS_RES_SHEAR, FS_RES_MEMBRANE = 1, 2, 3

function res_quantity(quantity)
    quantity in (:transverse_shear, :transverse, :shear) && return FS_RES_SHEAR
    quantity in (:membrane_force, :membrane) && return FS_RES_MEMBRANE
    return FS_RES_MOMENT    # :bending, :moment, :bending_moment, and the default :Cauchy
end

# location (1x3) and tangents (3x2) of point j of element i: the centroid and
# the edge Jacobian of a T3; Gauss point j of GaussRule(2,2) of a Q4
function point_geometry(geom0, conn, j, nen)
    X = geom0.values[collect(conn), :]
    if nen == 3
        return sum(X, dims = 1) ./ 3, hcat(X[2, :] - X[1, :], X[3, :] - X[1, :])
    end
    g = 0.577350269189626
    xi, eta = (j <= 2 ? -g : g), (iseven(j) ? g : -g)
    N = [(1 - xi) * (1 - eta), (1 + xi) * (1 - eta), (1 + xi) * (1 + eta), (1 - xi) * (1 + eta)] ./ 4
    dN = [-(1 - eta) -(1 - xi); (1 - eta) -(1 + xi); (1 + eta) (1 + xi); -(1 + eta) (1 - xi)] ./ 4
    return reshape(N' * X, 1, 3), X' * dN
end

for (T, etype, nen) in ((FEMMShellT3FF, FS_T3FF, 3), (FEMMShellQ4RS, FS_Q4RS, 4))
    @eval function inspectintegpoints(self::$T, geom0::NodalField{FFlt}, u::NodalField{TI},
        dT::NodalField{FFlt}, felist::FIntVec, inspector::F, idat, quantity = :Cauchy;
        context...) where {TI<:Number,F<:Function}
        @assert self._associatedgeometry == true
        fes = self.integdomain.fes
        outputcsys = self.mcsys
        for apair in pairs(context)
            sy, val = apair
            sy == :outputcsys && (outputcsys = val)
        end
        npe = $nen == 3 ? 1 : 4
        npt = count(fes) * npe
        cs = Array{Float64}(undef, 3, 3, npt)
        for i in 1:count(fes), j in 1:npe
            loc, J = point_geometry(geom0, fes.conn[i], j, $nen)
            updatecsmat!(outputcsys, loc, J, i, $nen == 3 ? 0 : j)
            cs[:, :, (i - 1) * npe + j] .= csmat(outputcsys)
        end
        ctx = context(self)
        upload!(ctx, self, $etype, geom0, nothing)
        out = Array{Float64}(undef, 3, npt)
        check(ctx, ccall((:fs_resultants, libflexshell), Cint,
            (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Float64}),
            ctx.h, res_quantity(quantity), Matrix{Float64}(u.values), cs, npt, out))
        for i in felist, j in 1:npe
            loc, _ = point_geometry(geom0, fes.conn[i], j, $nen)
            idat = inspector(idat, i, fes.conn[i], geom0.values[collect(fes.conn[i]), :],
                out[:, (i - 1) * npe + j], loc)
        end
        return idat
    end
end

# ---------------------------------------------------------------------------
# FEMMCorotBeam
# ---------------------------------------------------------------------------
# fs_beam_section (include/flexshell.h): the FESetL2Beam fields of one element
struct FsBeamSection
    A::Float64
    I1::Float64
    I2::Float64
    I3::Float64
    J::Float64
    A2s::Float64
    A3s::Float64
    x1x2_vector::NTuple{3,Float64}
end

function beam_upload!(ctx, femm::FEMMCorotBeam, geom0, u1, Rfield1, dchi, v1 = nothing)
    fes = femm.integdomain.fes
    d = delegateof(fes)
    conn = collect(reinterpret(Int, fes.conn))
    xyz = geom0.values
    check(ctx, ccall((:fs_mesh_set, libflexshell), Cint,
        (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}),
        ctx.h, FS_COROTBEAM, size(xyz, 1), xyz, count(fes), conn, C_NULL, dchi.dofnums))
    secs = [FsBeamSection(d.A[i], d.I1[i], d.I2[i], d.I3[i], d.J[i], d.A2s[i], d.A3s[i],
        Tuple(d.x1x2_vector[i])) for i in 1:count(fes)]
    check(ctx, ccall((:fs_beam_setup, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{FsBeamSection}, Float64, Float64, Float64),
        ctx.h, secs, femm.material.E, femm.material.nu, massdensity(femm.material)))
    check(ctx, ccall((:fs_beam_state_set, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        ctx.h, u1.values, Rfield1.values, v1 === nothing ? C_NULL : v1.values))
end

function beam_matrix(self, which, assembler, geom0, u1, Rfield1, dchi; mass_type = 1, v1 = nothing)
    ctx = context(self)
    beam_upload!(ctx, self, geom0, u1, Rfield1, dchi, v1)
    nnz = Ref{Int64}(0)
    check(ctx, ccall((:fs_beam_matrix, libflexshell), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Int64, Ref{Int64}),
        ctx.h, which, mass_type, asm_mode(assembler), nalldofs(dchi), nnz))
    return fetch_csc(ctx, nalldofs(dchi), nnz[])
end

stiffness(self::FEMMCorotBeam, assembler::AbstractSysmatAssembler, geom0::NodalField{Float64},
    u1::NodalField{Float64}, Rfield1::NodalField{Float64}, dchi::NodalField{TI}) where {TI} =
    beam_matrix(self, FS_BEAM_STIFFNESS, assembler, geom0, u1, Rfield1, dchi)
geostiffness(self::FEMMCorotBeam, assembler::AbstractSysmatAssembler, geom0::NodalField{Float64},
    u1::NodalField{Float64}, Rfield1::NodalField{Float64}, dchi::NodalField{TI}) where {TI} =
    beam_matrix(self, FS_BEAM_GEOSTIFFNESS, assembler, geom0, u1, Rfield1, dchi)
mass(self::FEMMCorotBeam, assembler::AbstractSysmatAssembler, geom0::NodalField{Float64},
    u1::NodalField{Float64}, Rfield1::NodalField{Float64}, dchi::NodalField{TI};
    mass_type = 1) where {TI} =
    beam_matrix(self, FS_BEAM_MASS, assembler, geom0, u1, Rfield1, dchi; mass_type = mass_type)
gyroscopic(self::FEMMCorotBeam, assembler::AbstractSysmatAssembler, geom0::NodalField{Float64},
    u1::NodalField{Float64}, Rfield1::NodalField{Float64}, v1::NodalField{Float64},
    dchi::NodalField{TI}; mass_type = 1) where {TI} =
    beam_matrix(self, FS_BEAM_GYROSCOPIC, assembler, geom0, u1, Rfield1, dchi;
        mass_type = mass_type, v1 = v1)

function restoringforce(self::FEMMCorotBeam, assembler::AbstractSysvecAssembler, geom0::NodalField{Float64},
    u1::NodalField{Float64}, Rfield1::NodalField{Float64}, dchi::NodalField{TI}) where {TI}
    ctx = context(self)
    beam_upload!(ctx, self, geom0, u1, Rfield1, dchi)
    F = zeros(nalldofs(dchi))
    check(ctx, ccall((:fs_beam_restoringforce, libflexshell), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}),
        ctx.h, length(F), F))
    return F
end

# uniform force intensity (ForceIntensity of a constant vector); loads varying
# per element go as a 3 x nelem array with per_element = 1
function distribloads_global(self::FEMMCorotBeam, assembler::AbstractSysvecAssembler,
    geom0::NodalField{Float64}, u1::NodalField{Float64}, Rfield1::NodalField{Float64},
    dchi::NodalField{TI}, fi) where {TI}
    ctx = context(self)
    beam_upload!(ctx, self, geom0, u1, Rfield1, dchi)
    q = Float64.(updateforce!(fi, zeros(0, 0), zeros(0, 0), 1, 0)[1:3])
    F = zeros(nalldofs(dchi))
    check(ctx, ccall((:fs_beam_distribloads_global, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Cint, Int64, Ptr{Float64}), ctx.h, q, 0, length(F), F))
    return F
end

# distributed surface loads of a shell element set: distribloads(femm::FEMMBase,
# assembler, geom, P, fi, m) of FinEtools on a T3 or Q4 set with TriRule(1, 3,
# 6) or GaussRule(2, 1..3); fi is evaluated on the host at the points
# fs_integration_points returns (updateforce!, as FinEtools does point by
# point), the element loop and the node sums run on the GPU.  A separate name:
# FEMMBase is FinEtools' own type.
function gpu_distribloads(self::FEMMBase, assembler::AbstractSysvecAssembler, geom::NodalField{Float64},
    P::NodalField{TI}, fi::ForceIntensity, m::Int) where {TI}
    ctx = context(self)
    fes = self.integdomain.fes
    nen = nodesperelem(fes)
    ir = self.integdomain.integration_rule
    rule = nen == 3 ? ir.npts : ir.order
    conn = collect(reinterpret(Int, fes.conn))
    xyz = geom.values
    # an L2 set (meshboundary edges) goes in as the library's two-node mesh type
    etype = nen == 2 ? FS_COROTBEAM : (nen == 3 ? FS_T3FF : FS_Q4RS)
    check(ctx, ccall((:fs_mesh_set, libflexshell), Cint,
        (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}),
        ctx.h, etype, size(xyz, 1), xyz, count(fes), conn, C_NULL, P.dofnums))
    npts = nen == 4 ? rule^2 : rule
    pts = zeros(9, count(fes) * npts)
    check(ctx, ccall((:fs_integration_points, libflexshell), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}),
        ctx.h, rule, pts))
    force = zeros(6, size(pts, 2))
    for k in 1:size(pts, 2)
        e, j = divrem(k - 1, npts)
        tangents = nen == 2 ? reshape(pts[4:6, k], 3, 1) : reshape(pts[4:9, k], 3, 2)
        force[:, k] .= updateforce!(fi, reshape(pts[1:3, k], 1, 3), tangents, fes.label[e + 1], j + 1)[1:6]
    end
    n = assembler isa SysvecAssemblerFBlock ? nfreedofs(P) : nalldofs(P)
    F = zeros(n)
    check(ctx, ccall((:fs_distribloads, libflexshell), Cint,
        (Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Int64, Int64, Ptr{Float64}),
        ctx.h, rule, m, force, size(force, 2), n, F))
    return F
end

end # module
