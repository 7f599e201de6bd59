"""
    FlexShellGPU

Julia-side binding of libflexshell.so (include/flexshell.h).  It adds methods
with the reference signatures of FinEtoolsFlexStructures.jl 3.6.4 so that
driver code calls them unchanged:

    stiffness(femm::FEMMShellT3FF, assembler, geom0, u1, Rfield1, dchi)
    mass(femm::FEMMShellT3FF, assembler, geom0, dchi)
    restoringforce(femm::FEMMShellT3FF, assembler, geom0, u1, Rfield1, dchi)

(and the same for FEMMShellQ4RS, FEMMShellT3FFComp, FEMMShellQ4RSComp; a
SysmatAssemblerSparseCSRSymm assembler gives a SparseMatrixCSR, the others a
SparseMatrixCSC),

    inspectintegpoints(femm, geom0, u, dT, felist, inspector, idat, quantity; outputcsys)

for FEMMShellT3FF and FEMMShellQ4RS, and for FEMMCorotBeam

    stiffness / geostiffness (femm, assembler, geom0, u1, Rfield1, dchi)
    mass(femm, assembler, geom0, u1, Rfield1, dchi; mass_type)
    gyroscopic(femm, assembler, geom0, u1, Rfield1, v1, dchi; mass_type)
    restoringforce(femm, assembler, geom0, u1, Rfield1, dchi)
    distribloads_global(femm, assembler, geom0, u1, Rfield1, dchi, fi)

and, for the distributed loads on a shell element set,

    gpu_distribloads(femm::FEMMBase, assembler, geom, P, fi, m)

the central-difference loop of the explicit examples on the FEMM's last
stiffness (plate_expl_examples.jl:61-94),

    gpu_cd_loop!(femm, M, ksi, omegad, U0, V0, tend, dt, force!, peek; ...)

and the shift-invert operator of a modal analysis (K - sigma M factorised on
the GPU), for an eigensolver that takes a user operator:

    gpu_shift_invert(femm, M_ff, sigma)

`associategeometry!` stays the reference's own; its normals are passed in.
The thickness is the IntegDomain's `otherdimension` at each element's
centroid (the T3FF loop evaluates it there, src/FEMMShellT3FFModule.jl:677;
the Q4RS loop per Gauss point, src/FEMMShellQ4RSModule.jl:924: a thickness
that varies inside a quadrilateral is taken at its centroid).
Not exercised in this repository (no Julia toolchain here); it is the
binding a maintainer adds next to the reference.
"""
module FlexShellGPU

using SparseArrays
using SparseMatricesCSR
using LinearAlgebra
using FinEtools
using FinEtoolsFlexStructures.FEMMShellT3FFModule: FEMMShellT3FF
using FinEtoolsFlexStructures.FEMMShellQ4RSModule: FEMMShellQ4RS
using FinEtoolsFlexStructures.FEMMShellT3FFCompModule: FEMMShellT3FFComp
using FinEtoolsFlexStructures.FEMMShellQ4RSCompModule: FEMMShellQ4RSComp
using FinEtoolsFlexStructures.AssemblyModule: SysmatAssemblerSparseCSRSymm
using FinEtoolsFlexStructures.CompositeLayupModule: laminate_stiffnesses!, laminate_transverse_stiffness!,
    laminate_inertia!, thickness
import FinEtoolsFlexStructures.FEMMShellT3FFModule: stiffness, mass
import FinEtoolsFlexStructures.FEMMShellQ4RSModule: stiffness, mass
import FinEtoolsFlexStructures.FEMMShellT3FFCompModule: stiffness, mass
import FinEtoolsFlexStructures.FEMMShellQ4RSCompModule: stiffness, mass
import FinEtoolsFlexStructures.FEMMShellT3FFModule: inspectintegpoints
import FinEtoolsFlexStructures.FEMMShellQ4RSModule: inspectintegpoints
using FinEtoolsFlexStructures.FEMMCorotBeamModule: FEMMCorotBeam
import FinEtoolsFlexStructures.FEMMCorotBeamModule: geostiffness, gyroscopic, restoringforce,
    distribloads_global

const libflexshell = get(ENV, "FLEXSHELL_LIB", "libflexshell.so")

const FS_T3FF, FS_T3FFCOMP, FS_Q4RS, FS_Q4RSCOMP, FS_COROTBEAM = 0, 1, 2, 3, 4
const FS_BEAM_STIFFNESS, FS_BEAM_GEOSTIFFNESS, FS_BEAM_MASS, FS_BEAM_GYROSCOPIC = 0, 1, 2, 3
const FS_FP64, FS_MIXED, FS_MIXED_COMP = 0, 1, 2
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

# fs_layup_group (include/flexshell.h)
struct FsLayupGroup
    A::NTuple{9,Float64}
    B::NTuple{9,Float64}
    D::NTuple{9,Float64}
    H::NTuple{4,Float64}
    csmat::NTuple{9,Float64}
    thickness::Float64
    mass_density::Float64
    moi_density::Float64
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

is_layered(femm) = femm isa FEMMShellT3FFComp || femm isa FEMMShellQ4RSComp

# element centroid (1 x 3) and the edge Jacobian J0 = [x2 - x1, x3 - x1] (3 x 2)
function centroid_and_J0(geom0, c)
    X = geom0.values[collect(c), :]
    return sum(X, dims = 1) ./ size(X, 1), hcat(X[2, :] - X[1, :], X[3, :] - X[1, :])
end

# the assembly order of a layered FEMM (layup group by layup group,
# src/FEMMShellT3FFCompModule.jl:600-606) and its groups: one per layup whose
# csys is constant, one per element of a layup whose csys varies (its matrix
# evaluated at the element's centroid, as the element loop does)
function layup_tables(femm, geom0)
    fes = femm.integdomain.fes
    order = Int64[]
    groups = FsLayupGroup[]
    egroup = zeros(Int32, count(fes))
    A, B, D, H = zeros(3, 3), zeros(3, 3), zeros(3, 3), zeros(2, 2)
    for (layup, eset) in femm.layup_groups
        laminate_stiffnesses!(layup, A, B, D)
        laminate_transverse_stiffness!(layup, H)
        md, mi = laminate_inertia!(layup)
        mk(cs) = FsLayupGroup(Tuple(vec(A)), Tuple(vec(B)), Tuple(vec(D)), Tuple(vec(H)), Tuple(vec(cs)),
            thickness(layup), md, mi)
        if layup.csys.isconstant
            push!(groups, mk(csmat(layup.csys)))
            egroup[eset] .= length(groups) - 1
        else
            for i in eset
                loc, J0 = centroid_and_J0(geom0, fes.conn[i])
                updatecsmat!(layup.csys, loc, J0, i, 0)
                push!(groups, mk(copy(csmat(layup.csys))))
                egroup[i] = length(groups) - 1
            end
        end
        append!(order, eset)
    end
    return order, groups, egroup
end

# per-element thickness: otherdimension at the element centroid
function element_thickness(femm, geom0)
    fes = femm.integdomain.fes
    nen = nodesperelem(fes)
    Nc = fill(1.0 / nen, nen, 1)
    t = zeros(count(fes))
    for i in 1:count(fes)
        loc, _ = centroid_and_J0(geom0, fes.conn[i])
        t[i] = femm.integdomain.otherdimension(loc, fes.conn[i], Nc)
    end
    return t
end

function upload!(ctx, femm, etype, geom0, dchi)
    fes = femm.integdomain.fes
    conn = collect(reinterpret(Int, fes.conn))          # nen per element, 1-based
    xyz = geom0.values                                  # nnodes x 3, column-major
    layered = is_layered(femm)
    order, groups, egroup = layered ? layup_tables(femm, geom0) : (Int64[], FsLayupGroup[], Int32[])
    check(ctx, ccall((:fs_mesh_set, libflexshell), Cint,
        (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}),
        ctx.h, etype, size(xyz, 1), xyz, count(fes), conn, layered ? order : C_NULL,
        dchi === nothing ? C_NULL : dchi.dofnums))
    Dps, Dt = layered ? (Matrix(1.0I, 3, 3), Matrix(1.0I, 2, 2)) : femm_material_matrices(femm)
    rho = layered ? 0.0 : massdensity(femm.material)
    tsf = (etype == FS_T3FF || etype == FS_T3FFCOMP) ? femm.transv_shear_formulation : 0
    p = FsShellParams(tsf, 0, femm.drilling_stiffness_scale, femm.threshold_angle,
        stab_coefficient(femm.stab_fun), Tuple(vec(Dps)), Tuple(vec(Dt)), rho, 0.0)
    th = layered ? C_NULL : element_thickness(femm, geom0)
    check(ctx, ccall((:fs_params_set, libflexshell), Cint, (Ptr{Cvoid}, Ref{FsShellParams}, Ptr{Float64}),
        ctx.h, p, th))
    if layered
        check(ctx, ccall((:fs_layups_set, libflexshell), Cint, (Ptr{Cvoid}, Int32, Ptr{FsLayupGroup}, Ptr{Int32}),
            ctx.h, length(groups), groups, egroup))
    end
    # normals from the reference's associategeometry! (honours a user mcsys)
    check(ctx, ccall((:fs_normals_set, libflexshell), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{UInt8}),
        ctx.h, femm._normals, UInt8.(femm._normal_valid)))
end

femm_material_matrices(femm) =
    FinEtoolsFlexStructures.FEMMShellT3FFModule._shell_material_stiffness(femm.material)

# the last matrix as the assembler's result type: the symmetric matrix's CSC
# arrays are also its CSR arrays, so SysmatAssemblerSparseCSRSymm
# (src/AssemblyModule.jl:47-53) gets them as a SparseMatrixCSR
function fetch_matrix(ctx, n, nnz, assembler)
    colptr = Vector{Int64}(undef, n + 1)
    rowval = Vector{Int64}(undef, nnz)
    nzval = Vector{Float64}(undef, nnz)
    check(ctx, ccall((:fs_matrix_copy, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}), ctx.h, colptr, rowval, nzval))
    assembler isa SysmatAssemblerSparseCSRSymm && return SparseMatrixCSR{1}(n, n, colptr, rowval, nzval)
    return SparseMatrixCSC(n, n, colptr, rowval, nzval)
end
fetch_csc(ctx, n, nnz) = fetch_matrix(ctx, n, nnz, nothing)

const SHELLS = ((FEMMShellT3FF, FS_T3FF), (FEMMShellQ4RS, FS_Q4RS),
    (FEMMShellT3FFComp, FS_T3FFCOMP), (FEMMShellQ4RSComp, FS_Q4RSCOMP))

for (T, etype) in SHELLS
    @eval function stiffness(self::$T, assembler::ASS, geom0::NodalField{Float64},
        u1::NodalField{TI}, Rfield1::NodalField{TI}, dchi::NodalField{TI};
        precision = FS_FP64) where {ASS<:AbstractSysmatAssembler,TI<:Number}
        @assert self._associatedgeometry == true
        ctx = context(self)
        upload!(ctx, self, $etype, geom0, dchi)
        nnz = Ref{Int64}(0)
        check(ctx, ccall((:fs_stiffness, libflexshell), Cint, (Ptr{Cvoid}, Cint, Cint, Int64, Ref{Int64}),
            ctx.h, precision, asm_mode(assembler), nalldofs(dchi), nnz))
        return fetch_matrix(ctx, nalldofs(dchi), nnz[], assembler)
    end
    @eval function mass(self::$T, assembler::A, geom0::NodalField{Float64},
        dchi::NodalField{TI}) where {A<:AbstractSysmatAssembler,TI<:Number}
        @assert self._associatedgeometry == true
        ctx = context(self)
        upload!(ctx, self, $etype, geom0, dchi)
        nnz = Ref{Int64}(0)
        check(ctx, ccall((:fs_mass, libflexshell), Cint, (Ptr{Cvoid}, Cint, Int64, Ref{Int64}),
            ctx.h, asm_mode(assembler), nalldofs(dchi), nnz))
        return fetch_matrix(ctx, nalldofs(dchi), nnz[], assembler)
    end
    # -K U for the generalized displacements in dchi.values (translations and
    # rotations of every node through dchi.dofnums): the shells' restoring
    # force, which the reference has no method for (its explicit loop forms
    # E = K U, plate_expl_examples.jl:85); the sign of FEMMCorotBeam's
    # restoringforce (force on the nodes)
    @eval function restoringforce(self::$T, assembler::AbstractSysvecAssembler, geom0::NodalField{Float64},
        u1::NodalField{TI}, Rfield1::NodalField{TI}, dchi::NodalField{TI};
        precision = FS_FP64) where {TI<:Number}
        @assert self._associatedgeometry == true
        ctx = context(self)
        upload!(ctx, self, $etype, geom0, dchi)
        n = nalldofs(dchi)
        nnz = Ref{Int64}(0)
        check(ctx, ccall((:fs_stiffness, libflexshell), Cint, (Ptr{Cvoid}, Cint, Cint, Int64, Ref{Int64}),
            ctx.h, precision, FS_ASM_SPARSE, n, nnz))
        U = zeros(n)
        for k in eachindex(dchi.dofnums)
            d = dchi.dofnums[k]
            1 <= d <= n && (U[d] = dchi.values[k])
        end
        F = zeros(n)
        check(ctx, ccall((:fs_restoring_force, libflexshell), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
            ctx.h, U, F))
        return F
    end
end

# ---------------------------------------------------------------------------
# _cd_loop!(M, K, ksi, U0, V0, tend, dt, force!, peek)
# (examples/shells/dynamics/homogeneous/explicit/plate_expl_examples.jl:61-94)
# on the GPU, K the last stiffness assembled for `femm` (assemble it with
# stiffness(femm, ...) first): C = ksi 2 omegad diag(M), the same time-step
# adjustment, and force!(F, t) evaluated on the host at every step time once
# up front as F = g(t) Fmag (the examples' form): `force!` is called at t = 0
# to give Fmag, `g(t)` scales it (g = t -> 1: a constant load).  The state is
# copied back for peek(step, U, V, t) every `peek_every` steps.
# ---------------------------------------------------------------------------
function gpu_cd_loop!(femm, M, ksi, omegad, U0, V0, tend, dt, force!, peek;
    g = t -> 1.0, peek_every = 1, precision = FS_MIXED_COMP)
    ctx = context(femm)
    m = Vector{Float64}(vec(diag(M)))
    n = length(m)
    C = (ksi * 2 * omegad) .* m
    nsteps = Int64(round(tend / dt))
    if nsteps * dt < tend
        dt = tend / (nsteps + 1)
    end
    invMC = 1.0 ./ (m .+ (dt / 2) .* C)
    # the load first: an assembly in this context after fs_explicit_setup
    # (a force! that assembles) would end the explicit state
    Fmag = zeros(n)
    force!(Fmag, 0.0)
    mul = [Float64(g(k * dt)) for k in 0:nsteps]
    A0 = invMC .* (mul[1] .* Fmag)
    check(ctx, ccall((:fs_explicit_setup, libflexshell), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Float64), ctx.h, precision, invMC, C, dt))
    check(ctx, ccall((:fs_explicit_set_state, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), ctx.h, Vector{Float64}(U0),
        Vector{Float64}(V0), A0))
    check(ctx, ccall((:fs_explicit_set_load, libflexshell), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Int64), ctx.h, Fmag, mul, length(mul), 0))
    U, V, A = zeros(n), zeros(n), zeros(n)
    peek(0, Vector{Float64}(U0), Vector{Float64}(V0), 0.0)
    done = 0
    while done < nsteps
        k = min(max(peek_every, 1), nsteps - done)
        check(ctx, ccall((:fs_explicit_run, libflexshell), Cint, (Ptr{Cvoid}, Int64), ctx.h, k))
        done += k
        check(ctx, ccall((:fs_explicit_get_state, libflexshell), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), ctx.h, U, V, A))
        peek(done, U, V, done * dt)
    end
    return U, V, A
end

# ---------------------------------------------------------------------------
# Shift-invert operator of a modal analysis: x = (K - sigma M)^{-1} b with K
# the last stiffness assembled for `femm` (the free-free block, stiffness with
# nrows = nfreedofs) and the lumped mass M (its diagonal), factorised once on
# the GPU (fs_shift_factor); the returned function applies it
# (fs_shift_solve), for an eigensolver that accepts such an operator in place
# of eigs' own factorisation (test/test_composite_shell_dynamics.jl:70-76).
# ---------------------------------------------------------------------------
function gpu_shift_invert(femm, M, sigma)
    ctx = context(femm)
    m = Vector{Float64}(vec(diag(M)))
    kd = Ref{Int64}(0)
    check(ctx, ccall((:fs_shift_factor, libflexshell), Cint, (Ptr{Cvoid}, Float64, Ptr{Float64}, Ref{Int64}),
        ctx.h, sigma, m, kd))
    return function (b::AbstractVecOrMat)
        B = Matrix{Float64}(reshape(b, length(m), :))
        X = similar(B)
        check(ctx, ccall((:fs_shift_solve, libflexshell), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}),
            ctx.h, size(B, 2), B, X))
        return b isa AbstractVector ? vec(X) : X
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
