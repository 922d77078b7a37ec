"""
    SMGPU

Julia binding of libsmgpu.so for NuclearToolkit.jl's ShellModel path.

`SMGPU.main_sm(sntf, target_nuc, num_ev, target_J; lm=300, ls=20, tol=1e-8,
precision=:fp64)` has the arguments and the return value of
`NuclearToolkit.main_sm` (src/ShellModel/shellmodel_main.jl:89-281) for
`target_J = []`: it returns the lowest `num_ev` eigenvalues.  Parsing,
basis, jump tables, H·v and the thick-restart Lanczos run inside the library
(GPU); Julia only passes the file name and receives the energies.

Set `ENV["SMGPU_LIB"]` to the path of libsmgpu.so before loading the module.
"""
module SMGPU

const libsmgpu = get(ENV, "SMGPU_LIB", "libsmgpu.so")

const SMGPU_OK = Cint(0)
const SMGPU_ERR_NOCONV = Cint(-8)
const PRECISION = Dict(:fp64 => Cint(0), :mixed => Cint(1))

last_error(h::Ptr{Cvoid}) = unsafe_string(ccall((:smgpu_last_error, libsmgpu), Cstring, (Ptr{Cvoid},), h))

function check(rc::Cint, h::Ptr{Cvoid})
    rc == SMGPU_OK && return nothing
    error("libsmgpu error $(rc): $(last_error(h))")
end

"""Create a problem handle (readsmsnt + basis + jump tables on the GPU)."""
function create(sntf::AbstractString, target_nuc::AbstractString; precision::Symbol=:fp64)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:smgpu_problem_create_from_snt, libsmgpu), Cint,
               (Cstring, Cstring, Cint, Ref{Ptr{Cvoid}}), sntf, target_nuc, PRECISION[precision], ref)
    check(rc, C_NULL)
    return ref[]
end

destroy(h::Ptr{Cvoid}) = ccall((:smgpu_problem_destroy, libsmgpu), Cint, (Ptr{Cvoid},), h)

function mdim(h::Ptr{Cvoid})
    md = Ref{Clonglong}(0); nb = Ref{Cint}(0)
    check(ccall((:smgpu_dims, libsmgpu), Cint, (Ptr{Cvoid}, Ref{Clonglong}, Ref{Cint}, Ptr{Clonglong}),
                h, md, nb, C_NULL), h)
    return Int(md[])
end

"""twf .+= H * wf, the semantics of operate_H! (lanczos_methods.jl:153)."""
function operate_H!(h::Ptr{Cvoid}, wf::Vector{Float64}, twf::Vector{Float64})
    check(ccall((:smgpu_matvec, libsmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint, Cint),
                h, wf, twf, 1, 1), h)
    return nothing
end

function main_sm(sntf, target_nuc, num_ev, target_J; lm=300, ls=20, tol=1.e-8, max_restarts=10000,
                 precision::Symbol=:fp64, is_show=false)
    length(target_J) == 0 || error("SMGPU: target_J must be [] (J projection is not in the GPU library)")
    h = create(sntf, target_nuc; precision=precision)
    try
        n = min(num_ev, mdim(h))
        en = zeros(Float64, n)
        stats = zeros(Cint, 8)
        rc = ccall((:smgpu_solve, libsmgpu), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cint, Cdouble, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Cint}),
                   h, num_ev, lm, ls, tol, max_restarts, C_NULL, en, C_NULL, stats)
        rc == SMGPU_ERR_NOCONV && @warn "Lanczos not converged after $(max_restarts) restarts"
        rc == SMGPU_ERR_NOCONV || check(rc, h)
        print("En. "); foreach(x -> print(lpad(string(round(x, digits=4)), 10), " "), en); print("\n")
        is_show && println("matvecs $(stats[2]) restarts $(stats[3])")
        return en
    finally
        destroy(h)
    end
end

end # module
