classdef GPEtask2compGB300 < GPEtask2comp
    %GPEtask2compGB300 - GPEtask2comp whose groundstate_itp runs on a GB300
    %GPU through libgpe (gpe_mex 'create_spinor' context, 'itp_2comp').
    %
    % Drop-in for GPEtask2comp: construct it exactly like
    % GPEtask2comp(grid, {V1, V2}); g (2x2), N1, N2, M1, M2 and Ntotal keep
    % their meaning, and groundstate_itp (lib/@GPEtask2comp/groundstate_itp.m)
    % returns phi ({phi1, phi2}), MU1, MU2 and EE as the reference does,
    % with a scalar omega on 2D grids (its rotating branch).  Single-precision
    % grid axes run in complex FP32.
    %
    % UNVERIFIED: no MATLAB was available where this file was written; the
    % library calls it makes are covered by the Python tests of the same ABI.

    properties (Hidden, SetAccess = protected)
        gb300_handle = uint64(0)
        gb300_npts = 0          % values of a stacked [X1(:); X2(:)] array
        gb300_class = 'double'
    end

    methods
        function obj = GPEtask2compGB300(grid, trappot)
            obj@GPEtask2comp(grid, trappot);
            x = gather(grid.x);
            y = gather(grid.y);
            obj.gb300_class = class(x);
            if grid.ndims == 3
                z = gather(grid.z);
                n = [numel(x) numel(y) numel(z)];
                dx = double([x(2)-x(1), y(2)-y(1), z(2)-z(1)]);
                span = double([x(end)-x(1), y(end)-y(1), z(end)-z(1)]);
            else
                n = [numel(x) numel(y) 1];
                dx = double([x(2)-x(1), y(2)-y(1), 1]);
                span = double([x(end)-x(1), y(end)-y(1), 0]);
            end
            obj.gb300_npts = 2 * prod(n);
            obj.gb300_handle = gpe_mex('create_spinor', grid.ndims, n, dx, span, obj.gb300_class);
        end

        function delete(obj)
            if obj.gb300_handle ~= 0
                gpe_mex('destroy', obj.gb300_handle);
                obj.gb300_handle = uint64(0);
            end
        end

        function [phi, varargout] = groundstate_itp(task, dt, eps, phi)
            % @GPEtask2comp/groundstate_itp.m semantics, executed by libgpe.
            if ~isscalar(task.omega)
                error('gpe:omega', 'libgpe runs GPEtask2comp.groundstate_itp with a scalar omega');
            end
            V = task.getVtotal(0);
            if nargin <= 3
                phi = cellfun(@(x) task.grid.normalize(rand(size(V{1}), 'like', V{1}) + ...
                    1i * rand(size(V{1}), 'like', V{1})) ./ sqrt(2), cell(1, 2), 'UniformOutput', false);
            end
            ntot = task.Ntotal;
            if isempty(ntot)
                ntot = 0;
            end
            % the reference's iteration cap (groundstate_itp.m:136) as itp_max_iter
            gpe_mex('set_params', task.gb300_handle, 0, 0, 0, ntot, 0, 10, 500000, 50, 0, double(task.omega));
            gpe_mex('set_spinor_params', task.gb300_handle, double(task.g), 0, 0);
            gpe_mex('set_potential', task.gb300_handle, double(gather([V{1}(:); V{2}(:)])));
            gpe_mex('set_state', task.gb300_handle, complex(gather([phi{1}(:); phi{2}(:)])));
            [MU1, MU2, EE] = gpe_mex('itp_2comp', task.gb300_handle, dt, eps, nargout >= 4, ...
                double([task.N1 task.N2]), double([task.M1 task.M2]));
            s = gpe_mex('get_state', task.gb300_handle, task.gb300_class, [task.gb300_npts 1]);
            sz = size(task.grid.mesh.x);
            half = task.gb300_npts / 2;
            phi = {reshape(s(1:half), sz), reshape(s(half+1:end), sz)};
            if isa(task.grid.x, 'gpuArray')
                phi = cellfun(@gpuArray, phi, 'UniformOutput', false);
            end
            if nargout >= 2, varargout{1} = MU1; end
            if nargout >= 3, varargout{2} = MU2; end
            if nargout >= 4, varargout{3} = EE; end
            task.init_state = phi;
            task.current_state = phi;
        end
    end
end
